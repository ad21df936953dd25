"""Spin-orbital CCSD / CCSD-DIIS / (T) on the GPU (scess_ccsd_so_solve,
scess_ccsd_so_triples) against the restatement (oracle/ccsd_so.py) and the
reference's cross-checks (Tests.cpp:550-551, :575-577, :698-703)."""
import numpy as np
import pytest

import oracle
from scess_gb300.synthetic import convergent_sigma, make_workload
from tests.golden import PINS, load
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


def _chem(eri):
    return np.ascontiguousarray(np.asarray(eri).transpose(0, 2, 1, 3))


def test_antisymmetrised_integrals_bit_exact(gctx):
    d = load('h2o_sto3g')
    w = gctx.ccsd_so(_chem(d['eri']), d['eps'], d['nocc'], keep_ints=True)
    assert np.array_equal(w.mints, oracle.antisymmetrise_spin(_chem(d['eri'])))


@pytest.mark.parametrize('tag', ['h2_sto3g', 'h2o_sto3g'])
@pytest.mark.parametrize('diis', [True, False])
def test_spin_ccsd_matches_oracle_and_pins(gctx, tag, diis):
    d = load(tag)
    ref = oracle.ccsd_spin_orbital(_chem(d['eri']), d['eps'], d['nocc'], diis=diis)
    got = gctx.ccsd_so(_chem(d['eri']), d['eps'], d['nocc'], diis=diis)
    assert got.converged and ref.converged
    assert got.iterations == ref.iterations
    # DIIS solves near-singular systems once the errors are small, which
    # magnifies last-bit differences of the dot products
    assert abs(got.E_CCSD - ref.E_CCSD) < (1e-9 if diis else 1e-11)
    assert rel_err(got.t2, ref.t2) < 1e-7
    assert abs(got.E_CCSD - PINS[tag]['E_CCSD'][0]) < 2e-6


def test_spin_ccsd_t_matches_closed_shell_pin(gctx):
    d = load('h2o_sto3g')
    ref = oracle.ccsd_t_spin_orbital(_chem(d['eri']), d['eps'], d['nocc'])
    got = gctx.ccsd_so(_chem(d['eri']), d['eps'], d['nocc'], triples=True)
    assert abs(got.E_T - ref.E_T) < 1e-12
    assert abs(got.E_T - PINS['h2o_sto3g']['E_T'][0]) < 1e-7          # Tests.cpp:575-577


def test_spin_ccsd_t_ccpvdz(gctx):
    """H2O/cc-pVDZ (48 spin orbitals, three 10^3 38^3 tensors in (T)) against
    the restatement's values (tests/golden/spin_pins.json).  The solver stops at
    |dE| < 1e-6 as the reference's does, so E_CCSD sits within 2e-6 and E_(T)
    within 5e-7 of the tightly converged closed-shell pins."""
    import json
    import os
    from tests.golden import HERE
    pin = json.load(open(os.path.join(HERE, 'spin_pins.json')))['h2o_ccpvdz']
    d = load('h2o_ccpvdz')
    got = gctx.ccsd_so(_chem(d['eri']), d['eps'], d['nocc'], triples=True)
    assert got.converged and got.iterations == pin['iterations']
    assert abs(got.E_CCSD - pin['E_CCSD']) < 1e-10
    assert abs(got.E_T - pin['E_T']) < 1e-12
    assert abs(got.E_CCSD - PINS['h2o_ccpvdz']['E_CCSD'][0]) < 2e-6
    assert abs(got.E_T - PINS['h2o_ccpvdz']['E_T'][0]) < 5e-7


@pytest.mark.parametrize('o,v', [(3, 9), (4, 11)])
def test_spin_synthetic_matches_oracle(gctx, o, v):
    w = make_workload(o, v, seed=6, sigma=convergent_sigma(o, v))
    chem = _chem(w.eri())
    ref = oracle.ccsd_t_spin_orbital(chem, w.eps, o)
    got = gctx.ccsd_so(chem, w.eps, o, triples=True, keep_ints=True)
    assert ref.converged and got.converged
    assert got.iterations == ref.iterations
    assert abs(got.E_CCSD - ref.E_CCSD) < 1e-11
    assert rel_err(got.t1, ref.t1) < 1e-8
    assert rel_err(got.t2, ref.t2) < 1e-8
    assert abs(got.E_T - ref.E_T) < 1e-12
    # the standalone triples entry point on the oracle's amplitudes
    et = gctx.ccsd_so_triples(got.mints, w.eps, o, ref.t1, ref.t2)
    assert abs(et - oracle.spin_triples_correction(ref.t1, ref.t2, w.eps, ref.mints, 2 * o)) < 1e-13


def test_spin_python_mirror(gctx):
    import scess_gb300 as s
    d = load('h2o_sto3g')
    w = s.CCSD_DIIS(_chem(d['eri']), d['eps'], d['nocc'])
    F = np.diag(np.repeat(d['eps'], 2))
    o2 = 2 * d['nocc']
    et = s.CalculateTriplesCorrection(w, F, w.mints, o2, F.shape[0] - o2)
    assert abs(et - PINS['h2o_sto3g']['E_T'][0]) < 1e-7
