"""Torch float64 (CPU) restatement of the CCSD residual numerators, for autograd.

Test infrastructure.  The contraction list is ``UpdateAmplitudes``
(``src/Quantum/CC/RCCSD.cpp:101-233``) exactly as in ``oracle/rccsd.py``,
returning the numerators (t1new, t2new) before the division by the
denominators (:235-236), as functions of (t1, t2, eri) so that
``torch.autograd`` gives the reference vector-Jacobian products that the
GPU engine's hand-written adjoint is checked against.
"""
from __future__ import annotations

import numpy as np
import torch

_es = torch.einsum


def _blocks(eri, o):
    O, V = slice(0, o), slice(o, None)
    ovov = eri[O, O, V, V].permute(0, 2, 1, 3)      # RCCSD.cpp:55
    oovv = eri[O, V, O, V].permute(0, 2, 1, 3)      # :57
    ovvo = eri[O, V, V, O].permute(0, 2, 1, 3)      # :59
    ovvv = eri[O, V, V, V].permute(0, 2, 1, 3)      # :61
    ovoo = eri[O, O, V, O].permute(0, 2, 1, 3)      # :63
    oooo = eri[O, O, O, O]                          # :64
    vvvv = eri[V, V, V, V]                          # :65
    oovv_phys = eri[O, O, V, V]                     # :66
    L_oovv = 2.0 * oovv_phys - oovv_phys.permute(0, 1, 3, 2)   # :68-69
    L_ovov = 2.0 * ovov - ovov.permute(0, 3, 2, 1)             # :70
    return ovov, oovv, ovvo, ovvv, ovoo, oooo, vvvv, oovv_phys, L_oovv, L_ovov


def _pt(x):
    return x + x.permute(1, 0, 3, 2)


def residual_numerators(eri, o, t1, t2):
    """(t1new, t2new) of UpdateAmplitudes before the division (torch tensors)."""
    ovov, oovv, ovvo, ovvv, ovoo, oooo, vvvv, oovv_phys, L_oovv, L_ovov = _blocks(eri, o)
    tau = t2 + _es('ia,jb->ijab', t1, t1)
    Foo = _es('kcld,ilcd->ki', L_ovov, tau)
    Fvv = -_es('kcld,klad->ac', L_ovov, tau)
    Fov = _es('kcld,ld->kc', L_ovov, t1)
    t1n = _es('ac,ic->ia', Fvv, t1) - _es('ki,ka->ia', Foo, t1)
    t1n = t1n + 2.0 * _es('kc,kica->ia', Fov, t2) - _es('kc,ikca->ia', Fov, t2)
    t1n = t1n + _es('ki,ka->ia', _es('kc,ic->ki', Fov, t1), t1)
    t1n = t1n + 2.0 * _es('kcai,kc->ia', ovvo, t1) - _es('kiac,kc->ia', oovv, t1)
    t1n = t1n + 2.0 * _es('kdac,ikcd->ia', ovvv, tau) - _es('kcad,ikcd->ia', ovvv, tau)
    t1n = t1n - 2.0 * _es('lcki,klac->ia', ovoo, tau) + _es('kcli,klac->ia', ovoo, tau)

    tmp2 = -_es('kibc,ka->abic', oovv, t1) + ovvv.permute(1, 3, 0, 2)
    t2n = _pt(_es('abic,jc->ijab', tmp2, t1))
    tmp2 = _es('kcai,jc->akij', ovvo, t1) + ovoo.permute(1, 3, 0, 2)
    t2n = t2n - _pt(_es('akij,kb->ijab', tmp2, t1))
    t2n = t2n + oovv_phys
    Loo = Foo + 2.0 * _es('lcki,lc->ki', ovoo, t1) - _es('kcli,lc->ki', ovoo, t1)
    Lvv = Fvv + 2.0 * _es('kdac,kd->ac', ovvv, t1) - _es('kcad,kd->ac', ovvv, t1)
    Woooo = (oooo + _es('lcki,jc->klij', ovoo, t1) + _es('kclj,ic->klij', ovoo, t1)
             + _es('kcld,ijcd->klij', ovov, tau))
    Wvvvv = vvvv - _es('kdac,kb->abcd', ovvv, t1) - _es('kcbd,ka->abcd', ovvv, t1)
    Wvoov = (ovvo.permute(2, 0, 3, 1) + _es('kcad,id->akic', ovvv, t1)
             - _es('kcli,la->akic', ovoo, t1) - 0.5 * _es('ldkc,ilda->akic', ovov, t2)
             - 0.5 * _es('lckd,ilad->akic', ovov, t2) + _es('ldkc,ilad->akic', ovov, t2)
             - _es('lkci,la->akic', _es('ldkc,id->lkci', ovov, t1), t1))
    Wvovo = (oovv.permute(2, 0, 3, 1) + _es('kdac,id->akci', ovvv, t1)
             - _es('lcki,la->akci', ovoo, t1) - 0.5 * _es('lckd,ilda->akci', ovov, t2)
             - _es('lcki,la->akci', _es('lckd,id->lcki', ovov, t1), t1))
    t2n = t2n + _es('klij,klab->ijab', Woooo, tau) + _es('abcd,ijcd->ijab', Wvvvv, tau)
    t2n = t2n + _pt(_es('ac,ijcb->ijab', Lvv, t2)) - _pt(_es('ki,kjab->ijab', Loo, t2))
    tmp = 2.0 * _es('akic,kjcb->ijab', Wvoov, t2) - _es('akci,kjcb->ijab', Wvovo, t2)
    t2n = t2n + _pt(tmp) - _pt(_es('akic,kjbc->ijab', Wvoov, t2))
    t2n = t2n - _pt(_es('bkci,kjac->ijab', Wvovo, t2))
    return t1n, t2n


def residual_vjp(eri, o, t1, t2, g1, g2):
    """Reference VJP (numpy in, numpy out): (g_t1, g_t2, g_eri)."""
    E = torch.tensor(np.asarray(eri), dtype=torch.float64, requires_grad=True)
    T1 = torch.tensor(np.asarray(t1), dtype=torch.float64, requires_grad=True)
    T2 = torch.tensor(np.asarray(t2), dtype=torch.float64, requires_grad=True)
    r1, r2 = residual_numerators(E, o, T1, T2)
    loss = (r1 * torch.tensor(g1)).sum() + (r2 * torch.tensor(g2)).sum()
    loss.backward()
    return T1.grad.numpy(), T2.grad.numpy(), E.grad.numpy()


def _r3_torch(Y):
    """r3(Y)_ijk = 4Y_ijk + Y_kij + Y_jki - 2Y_kji - 2Y_ikj - 2Y_jik on the last three axes."""
    def tp(p):
        return Y.permute(0, 1, 2 + p[0], 2 + p[1], 2 + p[2])
    return (4.0 * Y + tp((1, 2, 0)) + tp((2, 0, 1)) - 2.0 * tp((2, 1, 0))
            - 2.0 * tp((0, 2, 1)) - 2.0 * tp((1, 0, 2)))


def triples_energy(eri, eps, o, t1, t2):
    """E_(T) of RCCSD_TriplesCorrection (RCCSD_T.cpp:17-168) as a torch function of
    (eri, t1, t2), in the batched per-``a`` form of ``oracle.rccsd_t.rccsd_triples_correction``
    (P/R/S/Q repack :29-56, raw w :62-68, the six terms of Symmetrise :78-106,
    V :70-75, r3 :152-154, degeneracy :135-139, denominators :155, factor 2 :167)."""
    O, V = slice(0, o), slice(o, None)
    P = eri[O, V, V, V].permute(0, 3, 2, 1)      # P(i,f,a,b) = eri(i, o+b, o+a, o+f)
    R = eri[O, O, V, O].permute(0, 3, 1, 2)      # R(i,j,m,a) = eri(i, m, o+a, j)
    S = eri[O, O, V, V]                          # S(i,j,a,b) = eri(i, j, o+a, o+b)
    Q = t2.permute(3, 1, 0, 2)                   # Q(f,j,k,c) = t2(k,j,c,f)
    v = P.shape[1]
    e = torch.as_tensor(np.asarray(eps), dtype=torch.float64)
    eo, ev = e[:o], e[o:]
    Dijk = eo[:, None, None] + eo[None, :, None] + eo[None, None, :]
    energy = torch.zeros((), dtype=torch.float64)
    for a in range(v):
        n = a + 1
        A1 = _es('ifb,fjkc->bcijk', P[:, :, a, :n], Q[:, :, :, :n])
        A1 = A1 - _es('ijm,mkbc->bcijk', R[:, :, :, a], t2[:, :, :n, :n])
        A2 = _es('ifb,fjkc->bcijk', P[:, :, :n, a], Q[:, :, :, :n])
        A2 = A2 - _es('ijmb,mkc->bcijk', R[:, :, :, :n], t2[:, :, a, :n])
        A3 = _es('ifbc,fjk->bcijk', P[:, :, :n, :n], Q[:, :, :, a])
        A3 = A3 - _es('ijmb,mkc->bcijk', R[:, :, :, :n], t2[:, :, :n, a])
        W = (A1 + A1.permute(1, 0, 2, 4, 3) + A2.permute(0, 1, 3, 2, 4)
             + A3.permute(0, 1, 4, 2, 3) + A2.permute(1, 0, 3, 4, 2)
             + A3.permute(1, 0, 4, 3, 2))
        Vt = (_es('i,jkbc->bcijk', t1[:, a], S[:, :, :n, :n])
              + _es('jb,ikc->bcijk', t1[:, :n], S[:, :, a, :n])
              + _es('kc,ijb->bcijk', t1[:, :n], S[:, :, a, :n]))
        r3 = _r3_torch(W + Vt)
        bb, cc = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
        deg = np.ones((n, n))
        deg[(bb == a) | (cc == bb)] = 2.0
        deg[cc == a] = 6.0
        wgt = torch.as_tensor(np.where(cc <= bb, 1.0 / deg, 0.0))
        d3 = Dijk[None, None] - (ev[a] + ev[:n, None] + ev[None, :n])[:, :, None, None, None]
        energy = energy + ((W * r3 / d3).sum(dim=(2, 3, 4)) * wgt).sum()
    return 2.0 * energy


def triples_vjp(eri, eps, o, t1, t2):
    """Reference gradient of E_(T) (numpy in, numpy out): (E_T, dE/dt1, dE/dt2, dE/deri)."""
    E = torch.tensor(np.asarray(eri), dtype=torch.float64, requires_grad=True)
    T1 = torch.tensor(np.asarray(t1), dtype=torch.float64, requires_grad=True)
    T2 = torch.tensor(np.asarray(t2), dtype=torch.float64, requires_grad=True)
    e_t = triples_energy(E, eps, o, T1, T2)
    e_t.backward()
    return float(e_t.detach()), T1.grad.numpy(), T2.grad.numpy(), E.grad.numpy()
