"""Build the C-ABI shared library ``libmbrime.so`` with nvcc for sm_103a.

Each translation unit is compiled in parallel into ``montblanc_gb300/_build``
and linked into ``montblanc_gb300/libmbrime.so`` (both git-ignored).  Only
nvcc and the CUDA runtime are needed: no CMake, no PyTorch extension
machinery.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libmbrime.so')
SOURCES = ('mb_api.cu', 'mb_stages.cu', 'mb_fused.cu', 'mb_tc.cu')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
         '-I', os.path.join(ROOT, 'include')]


def nvcc():
    exe = shutil.which('nvcc')
    if exe is None:
        cand = '/usr/local/cuda/bin/nvcc'
        if os.path.exists(cand):
            return cand
        raise RuntimeError('nvcc not found; the montblanc_gb300 CUDA library cannot be built')
    return exe


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(ROOT, 'include', 'montblanc_gb300.h'))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def build(force=False, verbose=False, extra_flags=()):
    """Compile the library if any source is newer than it; return its path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace('.cu', '.o'))
        cmd = [exe, *ARCH, *FLAGS, *extra_flags, '-c', os.path.join(CSRC, src), '-o', obj]
        if verbose:
            print(' '.join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on %s:\n%s%s' % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + '.tmp'
    cmd = [exe, *ARCH, '-shared', '-o', tmp, *objs, '-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s%s' % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose=True))
