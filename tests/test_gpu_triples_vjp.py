"""Gradient of E_(T) on the GPU (scess_rccsd_triples_vjp): against torch autograd
of the restated (T) energy and against central finite differences (step 1e-5,
64 seeded directions) of the GPU's own FP64 (T)."""
import numpy as np
import pytest
import torch

from oracle import autodiff
from scess_gb300.synthetic import convergent_sigma, make_workload
from tests.gpu_common import gctx, rel_err  # noqa: F401

pytestmark = pytest.mark.gpu


def _point(o, v, seed=3):
    return make_workload(o, v, seed=seed, with_amplitudes=True, sigma=convergent_sigma(o, v))


# (o, v, block size): one block, several blocks with padded virtuals (13 = 4+4+4+1)
@pytest.mark.parametrize('o,v,nb,g_e', [(3, 8, None, 1.0), (4, 13, 4, 1.0), (5, 18, 5, -2.5)])
def test_triples_vjp_matches_autograd(gctx, monkeypatch, o, v, nb, g_e):
    if nb:
        monkeypatch.setenv('SCESS_TUNE', f't_nb={nb}')
    w = _point(o, v)
    eri = w.eri()
    e_ref, r1, r2, re = autodiff.triples_vjp(eri, w.eps, o, w.t1, w.t2)
    e, g1, g2, ge = gctx.triples_vjp(eri, w.eps, o, w.t1, w.t2, g_e=g_e, want_integrals=True)
    assert abs(e - e_ref) <= 1e-10 * max(1.0, abs(e_ref))
    assert rel_err(g1, g_e * r1) < 1e-10
    assert rel_err(g2, g_e * r2) < 1e-10
    assert rel_err(ge, g_e * re) < 1e-10


def test_triples_vjp_central_differences_64_directions(gctx, monkeypatch):
    monkeypatch.setenv('SCESS_TUNE', 't_nb=4')
    o, v = 4, 14
    w = _point(o, v, seed=5)
    eri, t1, t2 = w.eri(), w.t1, w.t2
    _, g1, g2, ge = gctx.triples_vjp(eri, w.eps, o, t1, t2, want_integrals=True)
    rng = np.random.default_rng(17)
    h = 1e-5
    worst = 0.0
    # each block of the direction is scaled to the rms of the values it perturbs
    scale = [np.sqrt(np.mean(x ** 2)) for x in (t1, t2, eri)]
    for _ in range(64):
        d1, d2, de = (s * rng.standard_normal(x.shape) for s, x in zip(scale, (t1, t2, eri)))

        def f(s):
            return gctx.triples(eri + s * de, w.eps, o, t1 + s * d1, t2 + s * d2, precision='fp64')
        fd = (f(h) - f(-h)) / (2 * h)
        an = float((g1 * d1).sum() + (g2 * d2).sum() + (ge * de).sum())
        worst = max(worst, abs(fd - an) / max(abs(an), 1e-30))
    assert worst <= 1e-6, worst


def test_triples_vjp_df_factors_match_autograd(gctx, monkeypatch):
    monkeypatch.setenv('SCESS_TUNE', 't_nb=4')
    o, v = 3, 10
    w = _point(o, v, seed=9)
    B = torch.tensor(w.B, dtype=torch.float64, requires_grad=True)
    eri = torch.einsum('Qpr,Qqs->pqrs', B, B)
    T1 = torch.tensor(w.t1, dtype=torch.float64, requires_grad=True)
    T2 = torch.tensor(w.t2, dtype=torch.float64, requires_grad=True)
    e_ref = autodiff.triples_energy(eri, w.eps, o, T1, T2)
    e_ref.backward()
    e, g1, g2, gB = gctx.triples_vjp(eps=w.eps, nocc=o, t1=w.t1, t2=w.t2, B=w.B,
                                     want_integrals=True)
    assert abs(e - float(e_ref.detach())) <= 1e-10 * max(1.0, abs(e))
    assert rel_err(g1, T1.grad.numpy()) < 1e-10
    assert rel_err(g2, T2.grad.numpy()) < 1e-10
    assert rel_err(gB, B.grad.numpy()) < 1e-10


def test_triples_vjp_energy_matches_forward(gctx):
    o, v = 6, 25
    w = _point(o, v, seed=2)
    eri = w.eri()
    e, *_ = gctx.triples_vjp(eri, w.eps, o, w.t1, w.t2)
    assert abs(e - gctx.triples(eri, w.eps, o, w.t1, w.t2, precision='fp64')) <= 1e-12 * abs(e)


def test_triples_vjp_central_differences_64_directions_at_o10_v90(gctx):
    """The (T) VJP at the adjoint workload's size (o=10, v=90, DF factors,
    denominator-scaled amplitudes): 64 seeded directions over (t1, t2, B), each
    block scaled to the rms of what it perturbs, against central differences
    (step 1e-5) of the GPU's FP64 (T) from B: <= 1e-6 relative per direction for
    the FP64 adjoint, <= 1e-5 for the tensor-core adjoint (FP32 accumulation)."""
    o, v = 10, 90
    w = _point(o, v, seed=4)
    t1, t2, B = w.t1, w.t2, w.B
    grads = {p: gctx.triples_vjp(eps=w.eps, nocc=o, t1=t1, t2=t2, B=B, want_integrals=True,
                                 precision=p)[1:] for p in ('fp64', 'mixed')}
    rng = np.random.default_rng(29)
    h = 1e-5
    worst = {'fp64': 0.0, 'mixed': 0.0}
    scale = [np.sqrt(np.mean(x ** 2)) for x in (t1, t2, B)]
    for _ in range(64):
        d1, d2, dB = (s * rng.standard_normal(x.shape) for s, x in zip(scale, (t1, t2, B)))
        dB = 0.5 * (dB + dB.transpose(0, 2, 1))

        def f(s):
            return gctx.triples(None, w.eps, o, t1 + s * d1, t2 + s * d2, B=B + s * dB,
                                precision='fp64')
        fd = (f(h) - f(-h)) / (2 * h)
        for p, (g1, g2, gB) in grads.items():
            an = float((g1 * d1).sum() + (g2 * d2).sum() + (gB * dB).sum())
            worst[p] = max(worst[p], abs(fd - an) / max(abs(an), 1e-30))
    # FP64 adjoint: 1e-6; the tensor-core adjoint (FP32 accumulation): 1e-5
    assert worst['fp64'] <= 1e-6, worst
    assert worst['mixed'] <= 1e-5, worst


def test_triples_vjp_mixed_matches_fp64(gctx, monkeypatch):
    """The tensor-core (T) VJP against the FP64 one over several blocks."""
    monkeypatch.setenv('SCESS_TUNE', 't_nb=4')
    o, v = 5, 18
    w = _point(o, v, seed=6)
    eri = w.eri()
    ef, f1, f2, fe = gctx.triples_vjp(eri, w.eps, o, w.t1, w.t2, want_integrals=True)
    em, m1, m2, me = gctx.triples_vjp(eri, w.eps, o, w.t1, w.t2, want_integrals=True,
                                      precision='mixed')
    assert abs(em - ef) <= 1e-6 * abs(ef)
    assert rel_err(m1, f1) < 1e-5
    assert rel_err(m2, f2) < 1e-5
    assert rel_err(me, fe) < 1e-5
