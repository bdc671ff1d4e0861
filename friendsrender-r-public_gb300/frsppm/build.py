"""In-tree build of the native libraries (no CMake, one -gencode, parallel).

* ``libfrsppm.so`` (next to this package's ``csrc/``): the CUDA kernels for
  sm_103a and the C++ host library behind include/friendsrender.h.
* the oracle libraries, built by ``oracle/build_oracle.py``.
"""
from __future__ import annotations

import os
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, 'csrc')
BUILD = os.path.join(PKG_DIR, '_build')
LIB = os.path.join(PKG_DIR, 'libfrsppm.so')
CUDA_HOME = os.environ.get('CUDA_HOME', '/usr/local/cuda')
NVCC = os.path.join(CUDA_HOME, 'bin', 'nvcc')
GENCODE = '-gencode=arch=compute_103a,code=sm_103a'

# The parity-critical arithmetic relies on no FMA contraction and IEEE
# division / square root (the nvcc defaults besides --fmad).
NVCC_FLAGS = ['-O3', '-std=c++17', GENCODE, '-lineinfo', '--fmad=false', '-prec-div=true',
              '-prec-sqrt=true', '-ftz=false', '-Xcompiler', '-fPIC', '-Xcompiler', '-ffp-contract=off']
CXX_FLAGS = ['-O2', '-std=c++17', '-fPIC', '-ffp-contract=off', '-fno-fast-math',
             '-I' + os.path.join(CUDA_HOME, 'include')]

CU_SOURCES = ['fr_kernels.cu', 'fr_noalloc.cu', 'fr_exact_check.cu', 'fr_tc_check.cu', 'fr_guide.cu', 'fr_bvh_gpu.cu']
CXX_SOURCES = ['fr_host.cpp', 'fr_bvh.cpp', 'fr_png.cpp', 'fr_image_read.cpp', 'fr_ingest.cpp']


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh'))]
    headers.append(os.path.join(REPO, 'include', 'friendsrender.h'))
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + '.o')
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + ['-c', s, '-o', o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + '.o')
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(['g++'] + CXX_FLAGS + ['-c', s, '-o', o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for j in jobs]
    for j, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out)
        if p.returncode != 0:
            raise RuntimeError('build failed: %s\n%s' % (' '.join(j), out))
    if force or jobs or _newer(LIB, objs):
        link = [NVCC, GENCODE, '-shared', '-cudart', 'static', '-o', LIB] + objs
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed: %s\n%s%s' % (' '.join(link), r.stdout, r.stderr))
    return LIB


if __name__ == '__main__':
    print(build_library(force='--force' in sys.argv, verbose=True))
