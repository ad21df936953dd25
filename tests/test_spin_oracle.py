"""The spin-orbital restatement (oracle/ccsd_so.py) against the reference's own
cross-checks: spin-orbital CCSD_DIIS reproduces H2's CCSD energy
(Tests.cpp:550-551, 1e-6) and H2O/STO-3G's closed-shell CCSD energy
(:698-703, 1e-6); the spin-orbital (T) reproduces the closed-shell E_(T)
(:575-577, 1e-7)."""
import numpy as np
import pytest

import oracle
from oracle import ccsd_so
from tests.golden import PINS, load


def _chem(d):
    return np.ascontiguousarray(d['eri'].transpose(0, 2, 1, 3))


@pytest.mark.parametrize('tag', ['h2_sto3g', 'h2o_sto3g'])
def test_spin_ccsd_diis_matches_closed_shell_pins(tag):
    d = load(tag)
    w = oracle.ccsd_spin_orbital(_chem(d), d['eps'], d['nocc'], diis=True)
    assert w.converged
    assert abs(w.E_CCSD - PINS[tag]['E_CCSD'][0]) < 1e-6


def test_spin_ccsd_plain_converges_to_the_same_energy():
    d = load('h2o_sto3g')
    a = oracle.ccsd_spin_orbital(_chem(d), d['eps'], d['nocc'], diis=False)
    b = oracle.ccsd_spin_orbital(_chem(d), d['eps'], d['nocc'], diis=True)
    assert a.converged and b.converged
    assert b.iterations < a.iterations
    assert abs(a.E_CCSD - b.E_CCSD) < 2e-6


def test_spin_triples_matches_closed_shell_pin():
    d = load('h2o_sto3g')
    w = oracle.ccsd_t_spin_orbital(_chem(d), d['eps'], d['nocc'])
    assert abs(w.E_T - PINS['h2o_sto3g']['E_T'][0]) < 1e-7
    # the closed-shell restatement on its own converged amplitudes
    r = oracle.solve_rccsd_diis(d['eri'], d['eps'], d['nocc'])
    ref = oracle.rccsd_triples_correction(d['eri'], d['eps'], d['nocc'], r.t1, r.t2)
    assert abs(w.E_T - ref) < 1e-7


def test_antisymmetrised_integrals_symmetries():
    d = load('h2o_sto3g')
    g = oracle.antisymmetrise_spin(_chem(d))
    n = d['eps'].shape[0]
    assert g.shape == (2 * n,) * 4
    assert np.array_equal(g, -g.transpose(1, 0, 2, 3))
    assert np.array_equal(g, -g.transpose(0, 1, 3, 2))
    assert np.allclose(g, g.transpose(2, 3, 0, 1), atol=1e-12)
    # spin-forbidden: <a b || a' b'> with total spin changed vanishes
    spin = np.arange(2 * n) % 2
    bad = (spin[:, None, None, None] + spin[None, :, None, None]) != \
        (spin[None, None, :, None] + spin[None, None, None, :])
    assert np.all(g[bad] == 0.0)
    # alpha-beta block: <p q || r s> = (pr|qs) for p, r alpha and q, s beta
    chem = _chem(d)
    assert np.array_equal(g[0::2, 1::2, 0::2, 1::2], chem.transpose(0, 2, 1, 3))


def test_diis_partial_pivot_solve_matches_numpy():
    rng = np.random.default_rng(3)
    e = rng.standard_normal((5, 40))
    n = 5
    B = -np.ones((n + 1, n + 1))
    B[n, n] = 0
    B[:n, :n] = e @ e.T
    B[:n, :n] /= np.max(np.abs(B[:n, :n]))
    rhs = np.zeros(n + 1)
    rhs[n] = -1
    c = np.linalg.solve(B, rhs)
    assert abs(np.sum(c[:n]) - 1.0) < 1e-12
    assert ccsd_so.MAX_DIIS_VECS == 6 and ccsd_so.DIIS_START == 3


def test_spin_and_closed_shell_restatements_agree_on_synthetic_integrals():
    """Two independent restatements of the same physics: the spin-orbital
    solvers stop at |dE| < 1e-6, so energies agree to that level."""
    from scess_gb300.synthetic import convergent_sigma, make_workload
    o, v = 3, 9
    w = make_workload(o, v, seed=6, sigma=convergent_sigma(o, v))
    eri = w.eri()
    s = oracle.ccsd_t_spin_orbital(_chem({'eri': eri}), w.eps, o)
    r = oracle.solve_rccsd_diis(eri, w.eps, o)
    assert s.converged and r.converged
    assert abs(s.E_CCSD - r.E_CCSD) < 2e-6
    et = oracle.rccsd_triples_correction(eri, w.eps, o, r.t1, r.t2)
    assert abs(s.E_T - et) < 2e-6 * max(1.0, abs(et))
    # closed-shell t1 is the alpha block of the spin-orbital t1
    assert np.allclose(s.t1[0::2, 0::2], r.t1, atol=1e-5)


def test_committed_ccpvdz_spin_values_reproduce():
    """tests/golden/spin_pins.json (used by the GPU test) is what the
    restatement gives now (make_spin_pins.py)."""
    import json
    import os
    from tests.golden import HERE
    pin = json.load(open(os.path.join(HERE, 'spin_pins.json')))['h2o_ccpvdz']
    d = load('h2o_ccpvdz')
    w = oracle.ccsd_t_spin_orbital(_chem(d), d['eps'], d['nocc'])
    assert w.converged and w.iterations == pin['iterations']
    assert abs(w.E_CCSD - pin['E_CCSD']) < 1e-12
    assert abs(w.E_T - pin['E_T']) < 1e-14
