"""In-tree build of the sm_103a library (``pyiid_gb300/_lib/libpyiid_gb300.so``).

One translation unit (``csrc/capi.cu``) compiled with nvcc for
``-gencode arch=compute_103a,code=sm_103a``; the CUDA runtime is linked
statically so the library has no path dependence on the toolkit.
"""
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


def build(force=False, verbose=False):
    """Compile the library if any source is newer than it; return its path."""
    out = lib_path()
    deps = _sources()
    if (not force and os.path.exists(out) and
            os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps)):
        return out
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = out + '.tmp'
    cmd = [_nvcc(), *ARCH, '-O3', '-lineinfo', '-std=c++17',
           '-Xcompiler', '-fPIC', '-shared', '-cudart', 'static',
           '-o', tmp, os.path.join(CSRC, 'capi.cu')]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
        print(' '.join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc failed:\n' + res.stdout + res.stderr)
    if verbose:
        print(res.stderr)
    os.replace(tmp, out)
    return out


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
