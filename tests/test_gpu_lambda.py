"""GPU Lambda equations and unrelaxed one-particle density against the torch
oracle (oracle/lambda_rdm.py) and against central differences of the
re-solved CCSD energy with respect to the Fock matrix."""
import numpy as np
import pytest

from oracle import lambda_rdm as LR
from scess_gb300.synthetic import make_workload
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def system(gctx):
    o, v = 3, 8
    w = make_workload(o, v, seed=4)
    eri = w.eri()
    wfn = gctx.solve(eri, w.eps, o, energy_convergence=1e-13, amplitude_convergence=1e-11)
    return o, w, eri, wfn


def test_lambda_matches_oracle(gctx, system):
    o, w, eri, wfn = system
    l1, l2, res = gctx.lambda_solve(eri, w.eps, o, wfn.t1, wfn.t2, amplitude_convergence=1e-11)
    assert res.converged
    r1, r2 = LR.solve_lambda(eri, np.diag(w.eps), o, wfn.t1, wfn.t2)
    assert rel_err(l1, r1) < 1e-8
    assert rel_err(l2, r2) < 1e-8


def test_rdm1_matches_oracle_and_finite_differences(gctx, system):
    o, w, eri, wfn = system
    f = np.diag(w.eps)
    l1, l2, _ = gctx.lambda_solve(eri, w.eps, o, wfn.t1, wfn.t2, amplitude_convergence=1e-11)
    dm = gctx.rdm1(eri, w.eps, o, wfn.t1, wfn.t2, l1, l2)
    assert np.allclose(dm, dm.T, atol=1e-14)
    ref = LR.rdm1(eri, f, o, wfn.t1, wfn.t2, l1, l2)
    assert rel_err(dm, ref) < 1e-10
    h = 1e-5
    for (p, q) in [(0, 0), (0, 2), (1, 5), (4, 9), (6, 6), (2, 10)]:
        S = np.zeros_like(f)
        S[p, q] = S[q, p] = 1.0
        Ep, _, _ = LR.solve_ccsd(eri, f + h * S, o)
        Em, _, _ = LR.solve_ccsd(eri, f - h * S, o)
        fd = (Ep - Em) / (2 * h)
        an = float((dm * S).sum())
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3), (p, q, fd, an)


def test_lambda_mixed_close_to_fp64(gctx):
    from scess_gb300.synthetic import convergent_sigma
    o, v = 10, 90
    w = make_workload(o, v, seed=0, sigma=convergent_sigma(o, v))
    eri = w.eri()
    wfn = gctx.solve(eri, w.eps, o)
    f1, f2, rf = gctx.lambda_solve(eri, w.eps, o, wfn.t1, wfn.t2)
    m1, m2, rm = gctx.lambda_solve(eri, w.eps, o, wfn.t1, wfn.t2, precision='mixed',
                                   amplitude_convergence=1e-7)
    assert rf.converged and rm.converged
    assert rel_err(m2, f2) < 1e-4
