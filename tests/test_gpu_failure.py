"""Failure handling of the drop-in calls, made on the host or by a bounded wait
that runs out; none of these tests faults, traps or hangs the GPU.

* the call's time limit (options.time_limit_s) ends a solve with
  SCESS_ERR_TIMEOUT at the reference's poll point (RCCSD.cpp:346);
* a context's device-memory cap makes an allocation fail with SCESS_ERR_OOM as
  a full device would, and the context stays usable;
* a tensor-core launch whose operand stage is never filled gives up its
  bounded wait: the call returns SCESS_ERR_CUDA and the next call is correct.
"""
import numpy as np
import pytest

import oracle
from scess_gb300 import cc
from scess_gb300.synthetic import make_workload
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def small():
    w = make_workload(5, 19, seed=0)
    eri = w.eri()
    return w, eri, oracle.solve_rccsd_diis(eri, w.eps, 5)


def test_time_limit_gives_timeout_and_the_context_recovers(gctx, small):
    w, eri, ref = small
    with pytest.raises(cc.ScessError) as e:
        gctx.solve(eri, w.eps, 5, time_limit_s=1e-9)
    assert e.value.status == cc.SCESS_ERR_TIMEOUT
    got = gctx.solve(eri, w.eps, 5)
    assert got.converged and abs(got.E_CCSD - ref.E_CCSD) < 1e-9


def test_memory_limit_gives_oom_and_the_context_recovers(gctx, small):
    w, eri, ref = small
    try:
        gctx.set_memory_limit(1 << 20)  # below the 4.5 MB of this eri alone
        with pytest.raises(cc.ScessError) as e:
            gctx.solve(eri, w.eps, 5)
        assert e.value.status == cc.SCESS_ERR_OOM
        assert 'limit' in str(e.value)
        assert gctx.memory_held() >= 0
    finally:
        gctx.set_memory_limit(0)
    got = gctx.solve(eri, w.eps, 5)
    assert got.converged and abs(got.E_CCSD - ref.E_CCSD) < 1e-9
    # a cap the solve fits in, above what the context already holds (its
    # workspaces persist between calls)
    cap = gctx.memory_held() + (1 << 30)
    try:
        gctx.set_memory_limit(cap)
        got = gctx.solve(eri, w.eps, 5, precision='mixed')
        assert got.converged and abs(got.E_CCSD - ref.E_CCSD) < 1e-6
        assert gctx.memory_held() <= cap
    finally:
        gctx.set_memory_limit(0)


def test_expired_pipeline_wait_returns_an_error_and_the_context_recovers(gctx):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((64, 96))
    B = rng.standard_normal((96, 80))
    ref = gctx.einsum('ik,kj->ij', A, B, precision='mixed', out_shape=(64, 80))
    assert rel_err(ref, A @ B) < 1e-6
    with pytest.raises(cc.ScessError):
        gctx.arm_wait_expiry(1 << 8)  # below the smallest bound accepted
    gctx.arm_wait_expiry(1 << 20)     # ~0.5 ms at 2 GHz
    with pytest.raises(cc.ScessError) as e:
        gctx.einsum('ik,kj->ij', A, B, precision='mixed', out_shape=(64, 80))
    assert e.value.status == cc.SCESS_ERR_CUDA
    assert 'wait expired' in str(e.value)
    again = gctx.einsum('ik,kj->ij', A, B, precision='mixed', out_shape=(64, 80))
    assert rel_err(again, ref) < 1e-12
