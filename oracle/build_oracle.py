"""ORACLE build recipe (test infrastructure only).

* oracle/_build/libfrport.so — the CPU restatement in oracle/port/ (g++,
  OpenMP, no fast-math, no FMA contraction), built on every machine; beside
  it libfrport64.so (the FP64 oracle) and libfrport_timing.so (the CPU
  baseline's build).
* oracle/_ref/frref — the reference's own SPPM path compiled from its sources
  by oracle/ref/Makefile; only when FR_REFERENCE_SRC names the reference's
  SPPM/SPPM directory and on x86-64 (the reference uses AVX intrinsics).
"""
from __future__ import annotations

import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
PORT_LIB = os.path.join(BUILD, 'libfrport.so')
PORT_SRC = os.path.join(HERE, 'port', 'sppm_port.cpp')
# The reference's SPPM/SPPM source directory; the reference is built only
# when this names one.
REF_SRC = os.environ.get('FR_REFERENCE_SRC', '')
REF_BIN = os.path.join(HERE, '_ref', 'frref')


# Builds of the restatement: the parity build (the reference's float
# arithmetic exactly: no fast-math, no FMA contraction), the FP64 oracle (the
# same source with FR_PORT_REAL=double) and the timing build for the CPU
# baseline, with the reference's own optimisation flags (SPPM/SPPM/makefile:
# -O2 -ffast-math -Ofast -fopenmp; its -mavx is x86-only and left out, so
# the same build runs on the Arm host).
PORT_BUILDS = {
    'f32': (PORT_LIB, ['-O2', '-fno-fast-math', '-ffp-contract=off']),
    'f64': (os.path.join(BUILD, 'libfrport64.so'), ['-O2', '-fno-fast-math', '-ffp-contract=off',
                                                     '-DFR_PORT_REAL=double']),
    'timing': (os.path.join(BUILD, 'libfrport_timing.so'), ['-O2', '-ffast-math', '-Ofast']),
}


def build_port(kind='f32', force=False):
    os.makedirs(BUILD, exist_ok=True)
    lib, flags = PORT_BUILDS[kind]
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(PORT_SRC):
        return lib
    cmd = ['g++', '-std=c++17', '-fopenmp', '-fPIC', '-shared'] + flags + [PORT_SRC, '-o', lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('oracle port build failed:\n' + r.stdout + r.stderr)
    return lib


def build_reference():
    if not REF_SRC or not os.path.isdir(REF_SRC) or platform.machine() not in ('x86_64', 'AMD64'):
        return None
    r = subprocess.run(['make', '-s', '-j8', 'REF=' + REF_SRC], cwd=os.path.join(HERE, 'ref'),
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('reference build failed:\n' + r.stdout + r.stderr)
    return REF_BIN


def build_all():
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(len(PORT_BUILDS)) as ex:
        list(ex.map(build_port, PORT_BUILDS))
    build_reference()


if __name__ == '__main__':
    build_all()
    print(PORT_LIB, REF_BIN if os.path.exists(REF_BIN) else '(reference not built here)')
