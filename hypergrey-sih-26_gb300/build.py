"""Builds the in-tree engine library boxqp/libboxqp.so for sm_103a.

The CUDA translation units and the host C++ units are compiled in parallel, then linked with
the static CUDA runtime, so the library needs nothing at run time but the NVIDIA driver.
Host code is compiled with -ffp-contract=off so the generator and the CSR builder round the
same way on x86-64 and aarch64.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / 'csrc'
OUT_DIR = PKG / '_build'
LIB = PKG / 'boxqp' / 'libboxqp.so'

CUDA_HOME = Path(os.environ.get('CUDA_HOME', '/usr/local/cuda'))
NVCC = str(CUDA_HOME / 'bin' / 'nvcc')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
CU_SOURCES = ['kernels.cu', 'engine.cu', 'box.cu', 'admm.cu']
CPP_SOURCES = ['planted.cpp', 'host.cpp']


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError('build step failed:\n' + ' '.join(cmd) + '\n' + proc.stdout + proc.stderr)
    return proc


def _stale(target, sources):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(force=False, verbose=False):
    """Compiles the engine if any source is newer than the library; returns the library path."""
    headers = list(CSRC.glob('*.cuh')) + list(CSRC.glob('*.h')) + [ROOT / 'include' / 'boxqp.h']
    sources = [CSRC / s for s in CU_SOURCES + CPP_SOURCES]
    if not force and not _stale(LIB, sources + headers + [Path(__file__)]):
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    inc = ['-I', str(ROOT / 'include'), '-I', str(CSRC)]
    jobs = []
    for s in CU_SOURCES:
        obj = OUT_DIR / (s + '.o')
        jobs.append([NVCC, *ARCH, '-lineinfo', '-O3', '-std=c++17', '-Xcompiler', '-fPIC,-ffp-contract=off',
                     *inc, '-c', str(CSRC / s), '-o', str(obj)])
    for s in CPP_SOURCES:
        obj = OUT_DIR / (s + '.o')
        jobs.append(['g++', '-O3', '-std=c++17', '-fPIC', '-ffp-contract=off', *inc, '-c', str(CSRC / s),
                     '-o', str(obj)])
    with ThreadPoolExecutor(max_workers=len(jobs)) as pool:
        for proc in pool.map(_run, jobs):
            if verbose and (proc.stdout or proc.stderr):
                print(proc.stdout + proc.stderr, file=sys.stderr)
    objs = [str(OUT_DIR / (s + '.o')) for s in CU_SOURCES + CPP_SOURCES]
    tmp = LIB.with_suffix('.so.tmp')
    _run([NVCC, *ARCH, '-shared', '-Xcompiler', '-fPIC', '-o', str(tmp), *objs, '-lpthread'])
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
