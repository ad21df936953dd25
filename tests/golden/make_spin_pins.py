"""Writes spin_pins.json: the spin-orbital restatement (oracle/ccsd_so.py) on
H2O/cc-pVDZ, too slow for the GPU tests to recompute (~30 s of NumPy).  The
reference's spin-orbital solver stops at |dE| < 1e-6, so its E_(T) sits
2.3e-7 from the tightly converged closed-shell pin; the GPU is compared with
these values instead.  Run from the repository root:
    python -m tests.golden.make_spin_pins"""
import json
import os

import numpy as np

import oracle
from tests.golden import HERE, load


def main():
    d = load('h2o_ccpvdz')
    chem = np.ascontiguousarray(d['eri'].transpose(0, 2, 1, 3))
    w = oracle.ccsd_t_spin_orbital(chem, d['eps'], d['nocc'])
    out = {'h2o_ccpvdz': {'E_CCSD': w.E_CCSD, 'E_T': w.E_T, 'iterations': w.iterations,
                          'converged': bool(w.converged)}}
    with open(os.path.join(HERE, 'spin_pins.json'), 'w') as f:
        json.dump(out, f, indent=1)
        f.write('\n')


if __name__ == '__main__':
    main()
