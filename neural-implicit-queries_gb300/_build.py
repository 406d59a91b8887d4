"""Build recipe for libniq.so (the CUDA kernels and their C ABI).

Each ``csrc/*.cu`` file is compiled for sm_103a by its own ``nvcc`` process (all in
parallel) and linked into ``libniq.so`` next to this file.  A rebuild happens only when
a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
BUILD_DIR = os.path.join(PKG, '_build')
LIB_PATH = os.path.join(PKG, 'libniq.so')

ARCH_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ARCH_FLAGS + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-I', INCLUDE,
                           '--expt-relaxed-constexpr']


def _nvcc():
    env = os.environ.get('NVCC')
    if env:
        return env
    found = shutil.which('nvcc')
    return found or '/usr/local/cuda/bin/nvcc'


def sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _inputs():
    return sources() + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(INCLUDE, '*.h'))


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def build(force=False, verbose=False, extra_flags=()):
    """Compile every CUDA source and link libniq.so; returns the library path."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + '.o')
        cmd = [nvcc] + NVCC_FLAGS + list(extra_flags) + ['-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-4000:]}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + '.tmp'
    cmd = [nvcc] + ARCH_FLAGS + ['-shared', '-o', tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == '__main__':
    import sys
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
