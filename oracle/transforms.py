"""NumPy float64 restatement of the AO->MO two-electron transform.

Test infrastructure.  Follows ``TransformTEI``
(``src/Quantum/Integrals/IntegralTransforms.cpp:32-59``): chemists' AO
integrals ``tei(mu,nu,kap,lam)`` are transformed one index at a time, lam with
D, kap with C, nu with B, mu with A (:44-55), and, when ``chem_to_phys``, the
result is reordered ``pqrs -> prqs`` (:57-59) so that ``out(p,q,r,s) = <pq|rs>``
is the physicists' eri the CCSD path reads (``RCCSD.cpp:399`` passes C four
times with ``true``).
"""
from __future__ import annotations

import numpy as np


def transform_tei(tei, A, B=None, C=None, D=None, chem_to_phys=False):
    B = A if B is None else B
    C = A if C is None else C
    D = A if D is None else D
    x = np.einsum('mnkl,ls->mnks', tei, D, optimize=True)     # (mu nu|kap lam) -> (mu nu|kap s)
    x = np.einsum('mnks,kr->mnrs', x, C, optimize=True)       # -> (mu nu|r s)
    x = np.einsum('mnrs,nq->mqrs', x, B, optimize=True)       # -> (mu q|r s)
    x = np.einsum('mqrs,mp->pqrs', x, A, optimize=True)       # -> (p q|r s)
    if chem_to_phys:
        x = x.transpose(0, 2, 1, 3)                           # out(p,r,q,s) = (pq|rs)
    return np.ascontiguousarray(x)
