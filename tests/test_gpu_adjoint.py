"""Hand-written GPU adjoint of the CCSD residual: against torch autograd of the
restated contractions and against central finite differences (step 1e-5)."""
import numpy as np
import pytest

from oracle import autodiff
from scess_gb300.synthetic import convergent_sigma, make_workload
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


def _point(o, v, seed=7):
    w = make_workload(o, v, seed=seed, sigma=convergent_sigma(o, v))
    rng = np.random.default_rng(seed)
    t1 = 0.02 * rng.standard_normal((o, v))
    t2 = 0.02 * rng.standard_normal((o, o, v, v))
    g1 = rng.standard_normal((o, v))
    g2 = rng.standard_normal((o, o, v, v))
    return w, t1, t2, g1, g2


@pytest.mark.parametrize('o,v', [(3, 7), (5, 19)])
def test_vjp_matches_autograd(gctx, o, v):
    w, t1, t2, g1, g2 = _point(o, v)
    eri = w.eri()
    rt1, rt2, re = autodiff.residual_vjp(eri, o, t1, t2, g1, g2)
    gt1, gt2, ge = gctx.residual_vjp(eri, o, t1, t2, g1, g2, want_integrals=True)
    assert rel_err(gt1, rt1) < 1e-11
    assert rel_err(gt2, rt2) < 1e-11
    assert rel_err(ge, re) < 1e-11


def test_vjp_central_differences_64_directions(gctx):
    o, v = 6, 30
    w, t1, t2, g1, g2 = _point(o, v)
    eri = w.eri()
    gt1, gt2, ge = gctx.residual_vjp(eri, o, t1, t2, g1, g2, want_integrals=True)
    rng = np.random.default_rng(11)
    h = 1e-5
    worst = 0.0
    # each block of the direction is scaled to the rms of the values it perturbs
    scale = [np.sqrt(np.mean(x ** 2)) for x in (t1, t2, eri)]
    for _ in range(64):
        d1, d2, de = (s * rng.standard_normal(x.shape) for s, x in zip(scale, (t1, t2, eri)))

        def f(s):
            r1, r2 = gctx.residual(eri + s * de, o, t1 + s * d1, t2 + s * d2)
            return float((r1 * g1).sum() + (r2 * g2).sum())
        fd = (f(h) - f(-h)) / (2 * h)
        an = float((gt1 * d1).sum() + (gt2 * d2).sum() + (ge * de).sum())
        worst = max(worst, abs(fd - an) / max(abs(an), 1e-30))
    assert worst <= 1e-6, worst


def test_vjp_df_factors_central_differences(gctx):
    o, v = 4, 12
    w, t1, t2, g1, g2 = _point(o, v)
    gt1, gt2, gB = gctx.residual_vjp(None, o, t1, t2, g1, g2, B=w.B, want_integrals=True)
    rng = np.random.default_rng(5)
    h = 1e-5
    for _ in range(8):
        dB = rng.standard_normal(w.B.shape)

        def f(s):
            from scess_gb300.synthetic import Workload
            ws = Workload(w.o, w.v, w.naux, w.eps, w.B + s * dB)
            r1, r2 = gctx.residual(ws.eri(), o, t1, t2)
            return float((r1 * g1).sum() + (r2 * g2).sum())
        fd = (f(h) - f(-h)) / (2 * h)
        an = float((gB * dB).sum())
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-12)


def test_vjp_mixed_close_to_fp64(gctx):
    # The mixed forward folds the T1 dressing of Wvvvv using tau(ijcd) = tau(jidc),
    # so the two forms agree on the closed-shell subspace t2(ijab) = t2(jiba):
    # compare there (symmetric t2 and cotangent, symmetrised t2 gradient).
    o, v = 10, 90
    w, t1, t2, g1, g2 = _point(o, v)
    t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))
    g2 = 0.5 * (g2 + g2.transpose(1, 0, 3, 2))
    eri = w.eri()
    f1, f2, _ = gctx.residual_vjp(eri, o, t1, t2, g1, g2, precision='fp64')
    m1, m2, _ = gctx.residual_vjp(eri, o, t1, t2, g1, g2, precision='mixed')
    sym = lambda x: 0.5 * (x + x.transpose(1, 0, 3, 2))  # noqa: E731
    assert rel_err(m1, f1) < 1e-5
    assert rel_err(sym(m2), sym(f2)) < 1e-5


def test_vjp_central_differences_64_directions_at_o10_v90(gctx):
    """The residual VJP at the adjoint workload's size (o=10, v=90, nmo=100,
    naux=300): 64 seeded directions over (t1, t2, B), each block scaled to the
    rms of what it perturbs, against central differences (step 1e-5) of the
    FP64 forward from B.  FP64 adjoint: <= 1e-6 relative per direction; the
    tensor-core adjoint (FP32 accumulation, split operands) is held to its
    contraction accuracy, <= 5e-5: with unit random cotangents its reverse
    contractions sum K ~ o v^2 terms of both signs, so their relative error is
    about sqrt(K) 2^-22 (measured 1.6e-5)."""
    o, v = 10, 90
    w, t1, t2, g1, g2 = _point(o, v)
    # on the closed-shell subspace t2(ijab) = t2(jiba), where the tensor-core
    # forward (its Wvvvv dressing uses tau(ijcd) = tau(jidc)) is the same function
    sym = lambda x: 0.5 * (x + x.transpose(1, 0, 3, 2))  # noqa: E731
    t2, g2 = sym(t2), sym(g2)
    B = w.B
    f64 = gctx.residual_vjp(None, o, t1, t2, g1, g2, B=B, want_integrals=True)
    mix = gctx.residual_vjp(None, o, t1, t2, g1, g2, B=B, want_integrals=True, precision='mixed')
    rng = np.random.default_rng(23)
    h = 1e-5
    scale = [np.sqrt(np.mean(x ** 2)) for x in (t1, t2, B)]
    worst = {'fp64': 0.0, 'mixed': 0.0}
    for _ in range(64):
        d1, d2, dB = (s * rng.standard_normal(x.shape) for s, x in zip(scale, (t1, t2, B)))
        d2 = sym(d2)
        dB = 0.5 * (dB + dB.transpose(0, 2, 1))  # B stays symmetric in (p, q)

        def f(s):
            r1, r2 = gctx.residual(None, o, t1 + s * d1, t2 + s * d2, B=B + s * dB)
            return float((r1 * g1).sum() + (r2 * g2).sum())
        fd = (f(h) - f(-h)) / (2 * h)
        for name, (gt1, gt2, gB) in (('fp64', f64), ('mixed', mix)):
            an = float((gt1 * d1).sum() + (gt2 * d2).sum() + (gB * dB).sum())
            worst[name] = max(worst[name], abs(fd - an) / max(abs(an), 1e-30))
    assert worst['fp64'] <= 1e-6, worst
    assert worst['mixed'] <= 5e-5, worst
