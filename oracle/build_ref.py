"""Compiles the oracle's C restatement (oracle/rccsd_t_ref.c) into oracle/_build/.

Test infrastructure: the shared library is the timed CPU baseline of (T) and
a second oracle for E_(T).  gcc -O3 -fopenmp, no machine-specific flags (the
same source builds on x86_64 and aarch64).

The reference itself cannot be compiled here: its CC code needs the Eigen
Tensor module (the Libraries/Eigen submodule is empty), Libint2, Boost,
LAPACK/LAPACKE, Libxc, fmt and the Dahlia engine, none of which is present.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
SRC = os.path.join(HERE, 'rccsd_t_ref.c')
LIB = os.path.join(BUILD, 'librccsd_t_ref.so')


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + '.tmp'
        subprocess.check_call(['gcc', '-O3', '-fopenmp', '-fPIC', '-shared', SRC, '-o', tmp])
        os.replace(tmp, LIB)
    return LIB


def load():
    lib = ctypes.CDLL(build())
    f = lib.scess_ref_triples
    dp = ctypes.POINTER(ctypes.c_double)
    f.argtypes = [dp, dp, ctypes.c_int64, ctypes.c_int64, dp, dp, ctypes.c_int64, ctypes.c_int64,
                  ctypes.c_int]
    f.restype = ctypes.c_double
    return lib


def triples(eri, eps, nocc, t1, t2, a_begin=0, a_end=None, nthreads=0) -> float:
    """E_(T) over leading virtuals [a_begin, a_end) with the C restatement."""
    import numpy as np
    lib = load()
    N = eps.shape[0]
    v = N - nocc
    a_end = v if a_end is None else a_end
    e = np.asfortranarray(eri, dtype=np.float64)
    t1f = np.asfortranarray(t1, dtype=np.float64)
    t2f = np.asfortranarray(t2, dtype=np.float64)
    ep = np.ascontiguousarray(eps, dtype=np.float64)
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    return lib.scess_ref_triples(p(e), p(ep), N, nocc, p(t1f), p(t2f), a_begin, a_end, nthreads)


if __name__ == '__main__':
    print(build())
