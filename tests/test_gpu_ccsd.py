"""CCSD on the GPU against the FP64 oracle and the reference's pins."""
import numpy as np
import pytest

import oracle
from scess_gb300.synthetic import convergent_sigma, make_workload
from tests.golden import PINS, load
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


def _amplitudes(o, v, seed=5):
    rng = np.random.default_rng(seed)
    t1 = 0.02 * rng.standard_normal((o, v))
    y = 0.02 * rng.standard_normal((o, o, v, v))
    return t1, 0.5 * (y + y.transpose(1, 0, 3, 2))


@pytest.mark.parametrize('o,v', [(3, 7), (5, 19), (6, 33)])
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('mixed', 2e-5)])
def test_residual_matches_oracle_update(gctx, o, v, precision, tol):
    w = make_workload(o, v, seed=1, sigma=convergent_sigma(o, v))
    eri = w.eri()
    t1, t2 = _amplitudes(o, v)
    ints = oracle.make_integral_blocks(eri, o)
    eia, eijab = oracle.rccsd.denominators(w.eps, o)
    rng = np.random.default_rng(9)
    drv = 0.01 * rng.standard_normal((o, o, v, v))
    drv = 0.5 * (drv + drv.transpose(1, 0, 3, 2))
    ref1, ref2 = oracle.update_amplitudes(ints, eia, eijab, drv, t1, t2)
    r1, r2 = gctx.residual(eri, o, t1, t2, t2_driver=drv, precision=precision)
    assert rel_err(r1 / eia, ref1) < tol
    assert rel_err(r2 / eijab, ref2) < tol


@pytest.mark.parametrize('tag', sorted(PINS))
def test_solve_fp64_reference_pins(gctx, tag):
    d = load(tag)
    w = gctx.solve(d['eri'], d['eps'], d['nocc'])
    ref = oracle.solve_rccsd_diis(d['eri'], d['eps'], d['nocc'])
    assert w.converged
    assert abs(w.E_CCSD - ref.E_CCSD) <= 1e-9
    assert w.iterations == ref.iterations
    val, tol = PINS[tag]['E_CCSD']
    assert abs(w.E_CCSD - val) <= tol
    assert rel_err(w.t2, ref.t2) < 1e-7


@pytest.mark.parametrize('o,v', [(5, 19), (10, 90)])
def test_solve_fp64_synthetic_matches_oracle(gctx, o, v):
    sig = 0.05 if (o, v) == (5, 19) else convergent_sigma(o, v)
    w = make_workload(o, v, seed=0, sigma=sig)
    eri = w.eri()
    ref = oracle.solve_rccsd_diis(eri, w.eps, o)
    got = gctx.solve(eri, w.eps, o)
    assert ref.converged and got.converged
    assert abs(got.E_CCSD - ref.E_CCSD) <= 1e-9
    # the per-iteration energies follow the oracle's (same DIIS semantics)
    n = min(len(ref.history), got.history.shape[0])
    h_ref = np.array([h[1] for h in ref.history[:n]])
    assert np.max(np.abs(got.history[:n, 0] - h_ref)) < 1e-8


def test_solve_df_equals_eri_path(gctx):
    w = make_workload(5, 19, seed=2)
    a = gctx.solve(w.eri(), w.eps, 5)
    b = gctx.solve(None, w.eps, 5, B=w.B)
    assert abs(a.E_CCSD - b.E_CCSD) < 1e-11


def test_solve_df_mixed_builds_blocks_on_tensor_cores(gctx):
    """Mixed DF solve: the integral blocks are contracted from B on the tensor
    cores (~3e-7 relative per integral); the energy stays within 1 uEh of the
    FP64 eri-path solve."""
    w = make_workload(8, 40, seed=5, sigma=convergent_sigma(8, 40))
    a = gctx.solve(w.eri(), w.eps, 8)
    b = gctx.solve(None, w.eps, 8, B=w.B, precision='mixed')
    assert b.converged
    assert abs(a.E_CCSD - b.E_CCSD) < 1e-6


@pytest.mark.parametrize('o,v', [(5, 19), (9, 44)])
def test_df_state_matches_eri_state(gctx, o, v):
    """A DF state contracts only the seven integral regions CCSD reads from B
    (no nmo^4 eri is allocated) and its (T) forms its slices from B: energies,
    amplitudes and E_(T) equal the eri state's."""
    w = make_workload(o, v, seed=4, sigma=convergent_sigma(o, v))
    sa = gctx.state(w.eri(), w.eps, o, max_iterations=200)
    gctx.profile(True)
    sb = gctx.state(None, w.eps, o, B=w.B, max_iterations=200)
    rep = gctx.profile_report()
    gctx.profile(False)
    assert 'host:state_build' in rep
    assert not any('eri_alloc' in k or 'eri_upload' in k for k in rep)
    ra, rb = sa.iterate(200)[0], sb.iterate(200)[0]
    assert ra.converged and rb.converged
    assert abs(ra.E_CCSD - rb.E_CCSD) < 1e-10
    t1a, t2a = sa.amplitudes()
    t1b, t2b = sb.amplitudes()
    assert rel_err(t2b, t2a) < 1e-8
    ea, eb = sa.triples()[0], sb.triples()[0]
    assert abs(ea - eb) < 1e-11
    em = sb.triples(precision='mixed')[0]
    assert abs(em - ea) < 1e-6  # the mixed-precision bar: 1 uEh
    sa.close()
    sb.close()


def test_f12_coupling_matches_oracle(gctx):
    o, v = 5, 19
    w = make_workload(o, v, seed=3)
    eri = w.eri()
    rng = np.random.default_rng(4)
    res = 0.003 * rng.standard_normal((o, o, v, v))
    res = 0.5 * (res + res.transpose(1, 0, 3, 2))
    en = 0.003 * rng.standard_normal((o, o, v, v))
    ref = oracle.solve_rccsd_diis(eri, w.eps, o, f12_residual=res, f12_energy=en)
    import scess_gb300 as s
    got = gctx.solve(eri, w.eps, o, f12=s.RCCSD_F12Coupling(res, en))
    assert got.converged
    assert abs(got.E_CCSD - ref.E_CCSD) < 1e-9
    assert abs(got.E_F12_Coupling - ref.E_F12_Coupling) < 1e-10


def test_solve_mixed_within_microhartree(gctx):
    o, v = 10, 90
    w = make_workload(o, v, seed=0, sigma=convergent_sigma(o, v))
    eri = w.eri()
    f = gctx.solve(eri, w.eps, o)
    m = gctx.solve(eri, w.eps, o, precision='mixed')
    assert m.converged and m.mixed_iterations > 0
    assert abs(m.E_CCSD - f.E_CCSD) <= 1e-6


def test_fp64_solve_is_bitwise_reproducible(gctx):
    w = make_workload(5, 19, seed=0)
    eri = w.eri()
    a = gctx.solve(eri, w.eps, 5)
    b = gctx.solve(eri, w.eps, 5)
    assert a.E_CCSD == b.E_CCSD and np.array_equal(a.t2, b.t2)


def test_nonconvergence_and_cancel(gctx):
    w = make_workload(5, 19, seed=0)
    eri = w.eri()
    r = gctx.solve(eri, w.eps, 5, max_iterations=2)
    assert not r.converged and r.E_CCSD == 0.0 and r.t1 is None and r.iterations == 2

    class Stopper:
        n = 0

        def ShouldStop(self):
            self.n += 1
            return self.n > 3
    r = gctx.solve(eri, w.eps, 5, thread=Stopper())
    assert not r.converged and r.iterations == 0


def test_invalid_inputs(gctx):
    import scess_gb300 as s
    w = make_workload(3, 7, seed=0)
    eri = w.eri()
    bad = eri.copy()
    bad[1, 2, 3, 4] = np.nan
    with pytest.raises(s.ScessError) as e:
        gctx.solve(bad, w.eps, 3)
    assert e.value.status == s.cc.SCESS_ERR_INVALID
    with pytest.raises(s.ScessError):
        gctx.solve(eri, w.eps, 10)


def test_console_log_lines(gctx):
    import io
    w = make_workload(3, 7, seed=0)
    buf = io.StringIO()
    gctx.solve(w.eri(), w.eps, 3, console=buf)
    text = buf.getvalue()
    assert 'CCSD(0): E(corr) =' in text and 'CCSD procedure converged' in text


def test_checkpoint_and_resume(gctx):
    w = make_workload(5, 19, seed=0)
    eri = w.eri()
    full = gctx.solve(eri, w.eps, 5, checkpoint=64)
    ck1, ck2 = full.checkpoints
    k = 6
    o, v = 5, 19
    t1 = ck1[k].reshape((o, v), order='F')
    t2 = ck2[k].reshape((o, o, v, v), order='F')
    res = gctx.solve(eri, w.eps, 5, t1_init=t1, t2_init=t2)
    assert res.converged and abs(res.E_CCSD - full.E_CCSD) < 1e-9
