"""ORACLE build recipe (test infrastructure only).

* oracle/_build/libfrport.so — the CPU restatement in oracle/port/ (g++,
  OpenMP, no fast-math, no FMA contraction), built on every machine.
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


def build_port(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(PORT_LIB) and os.path.getmtime(PORT_LIB) >= os.path.getmtime(PORT_SRC):
        return PORT_LIB
    cmd = ['g++', '-O2', '-std=c++17', '-fopenmp', '-fPIC', '-shared', '-fno-fast-math', '-ffp-contract=off',
           PORT_SRC, '-o', PORT_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('oracle port build failed:\n' + r.stdout + r.stderr)
    return PORT_LIB


def build_reference():
    if not REF_SRC or not os.path.isdir(REF_SRC) or platform.machine() not in ('x86_64', 'AMD64'):
        return None
    r = subprocess.run(['make', '-s', '-j8', 'REF=' + REF_SRC], cwd=os.path.join(HERE, 'ref'),
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('reference build failed:\n' + r.stdout + r.stderr)
    return REF_BIN


def build_all():
    build_port()
    build_reference()


if __name__ == '__main__':
    build_all()
    print(PORT_LIB, REF_BIN if os.path.exists(REF_BIN) else '(reference not built here)')
