"""Golden fixtures: real-molecule MO integrals (see make_molecules.py) and pins."""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# Known-answer energies of the reference's regression tests, src/SCESS/Tests.cpp:34-75
# (value, tolerance used there; checks at :570-577, :594-607, :684-704).
PINS = {
    'h2_sto3g': {'E_RHF': (-1.1175058851, 1e-8), 'E_MP2': (-0.0125038087, 1e-8),
                 'E_CCSD': (-0.0193419373, 1e-8)},
    'h2o_sto3g': {'E_RHF': (-74.9629832288, 1e-6), 'E_MP2': (-0.0355225667, 1e-7),
                  'E_CCSD': (-0.0494026324, 1e-7), 'E_T': (-0.0000673499, 1e-8)},
    'h2o_ccpvdz': {'E_RHF': (-76.0267859418, 1e-8), 'E_MP2': (-0.2039840885, 1e-8),
                   'E_CCSD': (-0.2133077024, 1e-7), 'E_T': (-0.0030574132, 1e-7)},
}


def unpack_unique(vals: np.ndarray, n: int) -> np.ndarray:
    """Expand unique chemists' (pq|rs) (p>=q, r>=s, pq>=rs) to physicists' <pq|rs>."""
    chem = np.empty((n, n, n, n))
    pq = [(p, q) for p in range(n) for q in range(p + 1)]
    x = 0
    for a, (p, q) in enumerate(pq):
        for (r, s) in pq[:a + 1]:
            v = vals[x]
            x += 1
            for (i, j) in ((p, q), (q, p)):
                for (k, l) in ((r, s), (s, r)):
                    chem[i, j, k, l] = v
                    chem[k, l, i, j] = v
    return np.ascontiguousarray(chem.transpose(0, 2, 1, 3))


def load(tag: str):
    """Returns dict(eri (phys, N^4), eps, nocc, E_RHF, and, when stored, ao_chem
    (AO (mu nu|kap lam), N^4) and C (AO x MO)) for a molecule fixture."""
    d = np.load(os.path.join(HERE, tag + '.npz'))
    n = int(d['nmo'])
    out = {'eri': unpack_unique(d['eri_unique'], n), 'eps': d['eps'], 'nocc': int(d['nocc']),
           'E_RHF': float(d['E_RHF'])}
    if 'ao_unique' in d.files:
        nao = d['C'].shape[0]
        out['ao_chem'] = np.ascontiguousarray(unpack_unique(d['ao_unique'], nao).transpose(0, 2, 1, 3))
        out['C'] = d['C']
    return out
