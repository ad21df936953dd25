"""The oracle against the reference's own known-answer energies (Tests.cpp:34-75)."""
import numpy as np
import pytest

import oracle
from oracle.rccsd_t import rccsd_triples_correction_literal
from tests.golden import PINS, load


@pytest.mark.parametrize('tag', sorted(PINS))
def test_rhf_fixture_matches_pin(tag):
    d = load(tag)
    ref, tol = PINS[tag]['E_RHF']
    assert abs(d['E_RHF'] - ref) <= tol


@pytest.mark.parametrize('tag', sorted(PINS))
def test_oracle_ccsd_pin(tag):
    d = load(tag)
    w = oracle.solve_rccsd_diis(d['eri'], d['eps'], d['nocc'])
    assert w.converged
    ref, tol = PINS[tag]['E_CCSD']
    assert abs(w.E_CCSD - ref) <= tol
    if 'E_T' in PINS[tag]:
        ref, tol = PINS[tag]['E_T']
        et = oracle.rccsd_triples_correction(d['eri'], d['eps'], d['nocc'], w.t1, w.t2)
        assert abs(et - ref) <= tol
        et_lit = rccsd_triples_correction_literal(d['eri'], d['eps'], d['nocc'], w.t1, w.t2)
        assert abs(et - et_lit) <= 1e-14


def test_fixture_symmetry():
    d = load('h2o_ccpvdz')
    eri = d['eri']
    # <pq|rs> = <qp|sr> = <rs|pq> (real orbitals)
    assert np.allclose(eri, eri.transpose(1, 0, 3, 2), atol=1e-14)
    assert np.allclose(eri, eri.transpose(2, 3, 0, 1), atol=1e-14)
    assert np.all(np.diff(d['eps']) >= 0)


def test_flop_formulas():
    # published algorithmic-work figures of the closed-shell path (FLOPs per CCSD iteration, per (T))
    assert abs(oracle.ccsd_flops(10, 90) / 2.91e10 - 1) < 5e-3
    assert abs(oracle.ccsd_flops(20, 180) / 1.735e12 - 1) < 5e-3
    assert abs(oracle.triples_flops(10, 90) / 1.51e11 - 1) < 5e-3
    assert abs(oracle.triples_flops(24, 240) / 1.022e14 - 1) < 5e-3
