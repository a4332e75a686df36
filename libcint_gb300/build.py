"""Build the CUDA library (libcintgpu.so, sm_103a) in-tree.

The product library is compiled with nvcc from the translation units under csrc/ in parallel;
output goes to libcint_gb300/_build/ (git-ignored).  No cmake and no torch build step: the library
is plain C-ABI and is loaded with ctypes.  (The CPU oracle the tests check against is built by the
repository's build entry, not here.)
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'libcintgpu.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-std=c++17', '-O3', '-lineinfo', '-Xcompiler', '-fPIC',
              '-I' + os.path.join(ROOT, 'include'), '-I' + CSRC]
SOURCES = ['rys_kernels.cu', 'rys_grad.cu', 'cintgpu_host.cpp', 'noalloc.cu', 'df_kernels.cu']
HEADERS = ['rys_kernels.h', 'rys_device.cuh', 'cintgpu_types.h', 'rys_tables.inc',
           'cintgpu_internal.h']


def _nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return 'nvcc'


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_library(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, 'include', 'cintgpu.h'))
    if not force and not _stale(LIB, deps):
        return LIB
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + '.o')
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ['-c', os.path.join(CSRC, src), '-o', obj]
        if verbose:
            print(' '.join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart']
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build(force=False):
    build_library(force=force)
    return LIB


if __name__ == '__main__':
    build(force='--force' in sys.argv)
    print(LIB)
