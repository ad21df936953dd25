"""AO->MO transform on the GPU (scess_transform_tei) against the oracle's
TransformTEI restatement, and chained into CCSD/(T) on H2O/cc-pVDZ against the
reference's pins (src/SCESS/Tests.cpp:34-75)."""
import numpy as np
import pytest

from oracle.transforms import transform_tei
from tests.golden import PINS, load
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


def test_transform_h2o_ccpvdz_matches_fixture_and_pins(gctx):
    d = load('h2o_ccpvdz')
    mo = gctx.transform_tei(d['ao_chem'], d['C'], chem_to_phys=True)
    assert np.max(np.abs(mo - d['eri'])) < 1e-12
    wfn = gctx.solve(mo, d['eps'], d['nocc'])
    et = gctx.triples(mo, d['eps'], d['nocc'], wfn.t1, wfn.t2)
    e_ccsd, tol_ccsd = PINS['h2o_ccpvdz']['E_CCSD']
    e_t, tol_t = PINS['h2o_ccpvdz']['E_T']
    assert abs(wfn.E_CCSD - e_ccsd) < tol_ccsd
    assert abs(et - e_t) < tol_t


@pytest.mark.parametrize('phys', [False, True])
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('mixed', 5e-6)])
def test_transform_four_matrices(gctx, phys, precision, tol):
    rng = np.random.default_rng(3)
    n = 24
    x = rng.standard_normal((n, n, n, n))
    tei = x + x.transpose(1, 0, 2, 3)
    A, B, C, D = (rng.standard_normal((n, k)) for k in (7, 11, 13, 17))
    ref = transform_tei(tei, A, B, C, D, chem_to_phys=phys)
    out = gctx.transform_tei(tei, A, B, C, D, chem_to_phys=phys, precision=precision)
    assert out.shape == ref.shape
    assert rel_err(out, ref) < tol


def test_transform_mixed_close_to_fp64_at_size(gctx):
    rng = np.random.default_rng(5)
    n, m = 64, 48
    x = rng.standard_normal((n, n, n, n)) * 0.01
    tei = x + x.transpose(1, 0, 3, 2)
    Cm = np.linalg.qr(rng.standard_normal((n, n)))[0][:, :m]
    f = gctx.transform_tei(tei, Cm, chem_to_phys=True, precision='fp64')
    g = gctx.transform_tei(tei, Cm, chem_to_phys=True, precision='mixed')
    assert rel_err(g, f) < 5e-6
