"""Closed-shell MP2 on the GPU (scess_mp2_energy, scess_mp2_energy_ao) against the
restatement and the reference's pins (Tests.cpp:37,42,51)."""
import numpy as np
import pytest

import oracle
from tests.golden import PINS, load
from tests.gpu_common import gctx  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('tag', ['h2_sto3g', 'h2o_sto3g', 'h2o_ccpvdz'])
def test_mp2_mo_pins(gctx, tag):
    d = load(tag)
    chem = np.ascontiguousarray(d['eri'].transpose(0, 2, 1, 3))
    e = gctx.mp2_energy(chem, d['eps'], d['nocc'])
    assert abs(e - oracle.mp2_energy(chem, d['eps'], d['nocc'])) < 1e-12
    val, tol = PINS[tag]['E_MP2']
    assert abs(e - val) <= tol


@pytest.mark.parametrize('tag', ['h2o_sto3g', 'h2o_ccpvdz'])
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-11), ('mixed', 1e-6)])
def test_mp2_ao(gctx, tag, precision, tol):
    d = load(tag)
    if 'ao_chem' not in d:
        pytest.skip('fixture has no AO integrals')
    e = gctx.mp2_energy_ao(d['ao_chem'], d['C'], d['eps'], d['nocc'], precision=precision)
    ref = oracle.mp2_energy_ao(d['ao_chem'], d['C'], d['eps'], d['nocc'])
    assert abs(e - ref) <= tol
    val, ptol = PINS[tag]['E_MP2']
    if precision == 'fp64':
        assert abs(e - val) <= ptol
