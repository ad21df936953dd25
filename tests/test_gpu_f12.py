"""CCSD-F12b coupling on the GPU (scess_f12b_coupling) against the restatement,
and the coupled solve it feeds."""
import numpy as np
import pytest

import oracle
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


def _tensors(N, o, seed):
    rng = np.random.default_rng(seed)
    eri = rng.standard_normal((N, N, N, N))
    f12 = 0.1 * rng.standard_normal((N, N, N, N))
    rep = 0.1 * rng.standard_normal((N, N, N, N))
    C = 0.01 * rng.standard_normal((o, o, N - o, N - o))
    return eri, f12, rep, C


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-13), ('mixed', 5e-6)])
@pytest.mark.parametrize('N,o', [(9, 3), (24, 5)])
def test_coupling_matches_restatement(gctx, precision, tol, N, o):
    eri, f12, rep, C = _tensors(N, o, 2)
    ref_res, ref_en = oracle.f12b_coupling(eri, f12, rep, C, o)
    got = gctx.f12b_coupling(eri, f12, rep, C, o, precision=precision)
    assert rel_err(got.residual, ref_res) < tol
    assert rel_err(got.energy, ref_en) < 1e-14


def test_coupled_solve_matches_oracle(gctx):
    """The coupling from the GPU drives the solver exactly as the restatement's
    coupling drives the oracle solve (CCSD_F12b.cpp:93-94)."""
    from scess_gb300.synthetic import make_workload
    o, v = 5, 19
    N = o + v
    w = make_workload(o, v, seed=3)
    eri = w.eri()
    rng = np.random.default_rng(9)
    f12 = 0.02 * rng.standard_normal((N, N, N, N))
    f12 = 0.5 * (f12 + f12.transpose(1, 0, 3, 2))  # <pq|rs> = <qp|sr>
    rep = 0.02 * rng.standard_normal((N, N, N, N))
    rep = 0.5 * (rep + rep.transpose(1, 0, 3, 2))
    C = 0.003 * rng.standard_normal((o, o, v, v))
    C = 0.5 * (C + C.transpose(1, 0, 3, 2))
    res, en = oracle.f12b_coupling(eri, f12, rep, C, o)
    ref = oracle.solve_rccsd_diis(eri, w.eps, o, f12_residual=res, f12_energy=en)
    cpl = gctx.f12b_coupling(eri, f12, rep, C, o)
    got = gctx.solve(eri, w.eps, o, f12=cpl)
    assert got.converged
    assert abs(got.E_CCSD - ref.E_CCSD) < 1e-9
    assert abs(got.E_F12_Coupling - ref.E_F12_Coupling) < 1e-9
