"""The MP2 restatement (RHF.cpp:267-345) against the reference's pins (Tests.cpp:37,42,51)."""
import pytest

import oracle
from tests.golden import PINS, load


@pytest.mark.parametrize('tag', ['h2_sto3g', 'h2o_sto3g', 'h2o_ccpvdz'])
def test_mp2_restatement_hits_pins(tag):
    d = load(tag)
    chem = d['eri'].transpose(0, 2, 1, 3)  # <pq|rs> -> (pr|qs)
    val, tol = PINS[tag]['E_MP2']
    assert abs(oracle.mp2_energy(chem, d['eps'], d['nocc']) - val) <= tol


@pytest.mark.parametrize('tag', ['h2o_sto3g'])
def test_mp2_ao_restatement_equals_mo(tag):
    d = load(tag)
    if 'ao_chem' not in d:
        pytest.skip('fixture has no AO integrals')
    chem = d['eri'].transpose(0, 2, 1, 3)
    e_mo = oracle.mp2_energy(chem, d['eps'], d['nocc'])
    e_ao = oracle.mp2_energy_ao(d['ao_chem'], d['C'], d['eps'], d['nocc'])
    assert abs(e_mo - e_ao) < 1e-10
