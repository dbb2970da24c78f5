"""Build recipe of the oracle's C restatements (test infrastructure).

gcc -O3 -fopenmp -shared -fPIC oracle/debye_ref.c -> oracle/_lib/libdebye_ref.so

The reference itself is pure Python (numba), so there is no reference C/C++
source to compile into oracle/_ref; its Python code is exercised by
tests/golden/make_golden.py instead.  No -march flags: the same source is
built on x86_64 here and on aarch64 GPU hosts.  The library is rebuilt unless
the stamp beside it equals the SHA-256 of the source and the command line.
"""
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, '_lib')
LIB = os.path.join(LIBDIR, 'libdebye_ref.so')
SRC = os.path.join(HERE, 'debye_ref.c')


def build(force=False):
    cc = os.environ.get('CC') or shutil.which('gcc') or 'cc'
    flags = ['-O3', '-fopenmp', '-shared', '-fPIC']
    h = hashlib.sha256(' '.join([cc, *flags]).encode())
    with open(SRC, 'rb') as f:
        h.update(f.read())
    digest, stamp = h.hexdigest(), LIB + '.sha256'
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + '.tmp'
    subprocess.run([cc, *flags, '-o', tmp, SRC, '-lm'], check=True)
    os.replace(tmp, LIB)
    with open(stamp, 'w') as f:
        f.write(digest + '\n')
    return LIB


if __name__ == '__main__':
    print(build(force=True))
