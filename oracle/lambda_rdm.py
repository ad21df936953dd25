"""Torch float64 oracle for the CCSD Lambda equations and the unrelaxed 1-RDM.

Test infrastructure.  The reference has no Lambda or density code; this
oracle defines them from its own residual.  ``UpdateAmplitudes``
(``RCCSD.cpp:101-233``) assumes canonical orbitals (f_ov = 0, diagonal
f_oo, f_vv; RCCSD.cpp:13-15, :109).  For a general Fock matrix f the same
closed-shell equations gain the terms written out in :func:`omega` (the form of
Hirata 2004 / PySCF ``rccsd.update_amps`` before it drops f_ov and the
off-diagonal Fock).  At f = diag(eps) they reduce to R(t) - D t.

* E(t; f) = 2 sum_ia f_ia t_ia + sum L_oovv tau
* Lagrangian L = E + lambda . Omega(t; f); Lambda equations dL/dt = 0 on the
  closed-shell subspace t2(ijab) = t2(jiba) (lambda2 likewise symmetric)
* unrelaxed one-particle density (correlation part, spin-summed, orbitals
  fixed): gamma_pq = dL/df_pq = dE_CCSD/df_pq
"""
from __future__ import annotations

import numpy as np
import torch

from .autodiff import residual_numerators

_es = torch.einsum


def omega(eri, o, t1, t2, foo, fvv, fov):
    """Closed-shell CCSD residual Omega(t; f) = R(t) + Fock terms (torch)."""
    r1, r2 = residual_numerators(eri, o, t1, t2)
    tmp = _es('kc,ic->ki', fov, t1)                     # sum_c f_kc t_ic
    r1 = r1 + _es('ac,ic->ia', fvv, t1) - _es('ki,ka->ia', foo, t1)
    r1 = r1 + 2.0 * _es('kc,kica->ia', fov, t2) - _es('kc,ikca->ia', fov, t2)
    r1 = r1 - _es('ki,ka->ia', tmp, t1) + fov          # (+1 -2) f_kc t_ka t_ic, + f_ia
    lvv = fvv - _es('kc,ka->ac', fov, t1)
    loo = foo + tmp
    x = _es('ac,ijcb->ijab', lvv, t2) - _es('ki,kjab->ijab', loo, t2)
    r2 = r2 + x + x.permute(1, 0, 3, 2)
    return r1, r2


def energy(eri, o, t1, t2, fov):
    ov = eri[:o, :o, o:, o:]
    L = 2.0 * ov - ov.permute(0, 1, 3, 2)
    tau = t2 + _es('ia,jb->ijab', t1, t1)
    return 2.0 * (fov * t1).sum() + (L * tau).sum()


def _split(f, o):
    return f[:o, :o], f[o:, o:], f[:o, o:]


def solve_ccsd(eri, f, o, tol=1e-13, maxit=300):
    """CCSD amplitudes for a general (symmetric) Fock matrix: Jacobi on Omega + DIIS."""
    from .rccsd import AmplitudeDIIS
    E_ = torch.tensor(eri)
    foo, fvv, fov = (torch.tensor(x) for x in _split(f, o))
    e = np.diag(f)
    v = f.shape[0] - o
    d1 = torch.tensor(e[:o, None] - e[None, o:])
    d2 = d1[:, None, :, None] + d1[None, :, None, :]
    t1 = torch.zeros((o, v), dtype=torch.float64)
    t2 = torch.zeros((o, o, v, v), dtype=torch.float64)
    diis = AmplitudeDIIS(8)
    E_last = None
    for it in range(maxit):
        r1, r2 = omega(E_, o, t1, t2, foo, fvv, fov)
        n1, n2 = t1 + r1 / d1, t2 + r2 / d2
        new = np.concatenate([n1.numpy().ravel(), n2.numpy().ravel()])
        old = np.concatenate([t1.numpy().ravel(), t2.numpy().ravel()])
        ext = diis.extrapolate(new, new - old) if it >= 2 else new
        if it < 2:
            diis.extrapolate(new, new - old)
        t1 = torch.tensor(ext[:o * v].reshape(o, v))
        t2 = torch.tensor(ext[o * v:].reshape(o, o, v, v))
        E = float(energy(E_, o, t1, t2, fov))
        if E_last is not None and abs(E - E_last) < tol and np.linalg.norm(new - old) < 1e-10:
            break
        E_last = E
    return E, t1.numpy(), t2.numpy()


def solve_lambda(eri, f, o, t1, t2, tol=1e-11, maxit=300):
    """lambda with dE/dt + (dOmega/dt)^T lambda = 0, by Jacobi sweeps with autograd VJPs."""
    E_ = torch.tensor(eri)
    foo, fvv, fov = (torch.tensor(x) for x in _split(f, o))
    e = np.diag(f)
    d1 = torch.tensor(e[:o, None] - e[None, o:])
    d2 = d1[:, None, :, None] + d1[None, :, None, :]
    T1 = torch.tensor(t1, requires_grad=True)
    T2 = torch.tensor(t2, requires_grad=True)
    gE1, gE2 = torch.autograd.grad(energy(E_, o, T1, T2, fov), (T1, T2))
    r1, r2 = omega(E_, o, T1, T2, foo, fvv, fov)
    l1, l2 = gE1 / d1, gE2 / d2
    for _ in range(maxit):
        j1, j2 = torch.autograd.grad((r1, r2), (T1, T2), (l1, l2), retain_graph=True)
        # t2 is constrained to t2(ijab) = t2(jiba): the stationarity condition is the
        # symmetric part of the gradient (the antisymmetric subspace is unstable)
        j2 = 0.5 * (j2 + j2.permute(1, 0, 3, 2))
        n1 = l1 + (gE1 + j1) / d1
        n2 = l2 + (gE2 + j2) / d2
        ch = float(torch.sqrt(((n1 - l1) ** 2).sum() + ((n2 - l2) ** 2).sum()))
        l1, l2 = n1, n2
        if ch < tol:
            break
    return l1.detach().numpy(), l2.detach().numpy()


def rdm1(eri, f, o, t1, t2, l1, l2):
    """gamma = dL/df as an N x N matrix, split symmetrically over (p,q) and (q,p)."""
    E_ = torch.tensor(eri)
    foo, fvv, fov = (torch.tensor(x, requires_grad=True) for x in _split(f, o))
    T1, T2 = torch.tensor(t1), torch.tensor(t2)
    r1, r2 = omega(E_, o, T1, T2, foo, fvv, fov)
    lag = energy(E_, o, T1, T2, fov) + (torch.tensor(l1) * r1).sum() + (torch.tensor(l2) * r2).sum()
    goo, gvv, gov = torch.autograd.grad(lag, (foo, fvv, fov))
    N = f.shape[0]
    g = np.zeros((N, N))
    g[:o, :o] = 0.5 * (goo.numpy() + goo.numpy().T)
    g[o:, o:] = 0.5 * (gvv.numpy() + gvv.numpy().T)
    g[:o, o:] = 0.5 * gov.numpy()
    g[o:, :o] = 0.5 * gov.numpy().T
    return g
