"""In-tree build of the sm_103a library (``pyiid_gb300/_lib/libpyiid_gb300.so``).

One translation unit (``csrc/capi.cu``) compiled with nvcc for
``-gencode arch=compute_103a,code=sm_103a``; the CUDA runtime is linked
statically so the library has no path dependence on the toolkit.

The library is rebuilt unless its stamp (``libpyiid_gb300.so.sha256`` beside
it) equals the SHA-256 of every source under ``csrc/``, the public header,
the nvcc command line and the nvcc version, so a library copied or checked
out next to edited sources is never reused.
"""
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
LIBDIR = os.path.join(HERE, '_lib')
LIBNAME = 'libpyiid_gb300.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'),
                 '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found (set NVCC or put nvcc on PATH)')


def _sources():
    deps = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith(('.cu', '.cuh', '.h'))]
    deps.append(os.path.join(REPO, 'include', 'pyiid_gb300.h'))
    return deps


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _flags():
    return [*ARCH, '-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
            '-shared', '-cudart', 'static']


def source_hash(nvcc=None):
    """SHA-256 over the sources (names and bytes), the nvcc flags and the
    nvcc version string."""
    h = hashlib.sha256()
    for d in _sources():
        h.update(os.path.relpath(d, REPO).encode() + b'\0')
        with open(d, 'rb') as f:
            h.update(f.read())
        h.update(b'\0')
    h.update(' '.join(_flags()).encode())
    nvcc = nvcc or _nvcc()
    res = subprocess.run([nvcc, '--version'], capture_output=True, text=True)
    h.update(res.stdout.encode())
    return h.hexdigest()


def stamp_path():
    return lib_path() + '.sha256'


def is_current(nvcc=None):
    """True when the built library's stamp matches the current sources."""
    out, st = lib_path(), stamp_path()
    if not (os.path.exists(out) and os.path.exists(st)):
        return False
    with open(st) as f:
        return f.read().strip() == source_hash(nvcc)


def build(force=False, verbose=False):
    """Compile the library unless its stamp matches the sources; return its
    path."""
    out = lib_path()
    nvcc = _nvcc()
    digest = source_hash(nvcc)
    if not force and os.path.exists(out) and os.path.exists(stamp_path()):
        with open(stamp_path()) as f:
            if f.read().strip() == digest:
                return out
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = out + '.tmp'
    cmd = [nvcc, *_flags(), '-o', tmp, os.path.join(CSRC, 'capi.cu')]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
        print(' '.join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc failed:\n' + res.stdout + res.stderr)
    if verbose:
        print(res.stderr)
    os.replace(tmp, out)
    with open(stamp_path() + '.tmp', 'w') as f:
        f.write(digest + '\n')
    os.replace(stamp_path() + '.tmp', stamp_path())
    return out


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
