"""Seeded synthetic closed-shell CC workloads with density-fitted integrals.

The inputs stand in for real-molecule integrals at sizes where no molecule is
at hand.  Draw order (NumPy ``default_rng`` PCG64, frozen):

1. ``e_occ = sort(U[-1.5, -0.3], o)``, ``e_vir = sort(U[0.2, 3.0], v)``;
2. ``X ~ N(0, sigma_B^2)`` (stated: sigma_B = 0.05) of shape (naux, N, N), naux = 3N; ``B[Q,p,q] =
   X[Q, min(p,q), max(p,q)]`` (symmetric in pq);
3. only for fixed-amplitude (T) workloads: ``x ~ N(0, 0.01^2)`` (o, v) then
   ``y ~ N(0, 0.01^2)`` (o, o, v, v); ``t1 = x * mean|D1| / |D1|``,
   ``t2 = (y + y^T)/2 * mean|D2| / |D2|`` (``y^T[i,j,a,b] = y[j,i,b,a]``).

The stated distribution (sigma_B = 0.05) is not a physical Hamiltonian: its
vvvv ladder operator has a coherent eigenvalue of about naux*v*sigma_B^2
(67 Eh at o=10, v=90), so the CCSD iteration diverges beyond the smallest
size.  ``convergent_sigma(o, v)`` gives the documented convergent variant: it
keeps naux*v*sigma_B^2 at its o=5, v=19 value (3.42), where the stated
distribution converges.  Every workload records which sigma it used.

Chemists' integrals are ``(pq|rs) = sum_Q B[Q,p,q] B[Q,r,s]``; the drop-in
``eri[p,q,r,s] = <pq|rs> = (pr|qs)`` (physicists' notation, occupied first).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Workload:
    o: int
    v: int
    naux: int
    eps: np.ndarray        # (N,) orbital energies, occupied first
    B: np.ndarray          # (naux, N, N) DF factors, symmetric in the last two
    t1: np.ndarray | None = None   # (o, v) fixed amplitudes for (T)-only runs
    t2: np.ndarray | None = None   # (o, o, v, v)
    sigma: float = 0.05

    @property
    def nmo(self) -> int:
        return self.o + self.v

    def eri(self) -> np.ndarray:
        """Full N^4 physicists' integrals, eri[p,q,r,s] = (pr|qs)."""
        N = self.nmo
        Bm = self.B.reshape(self.naux, N * N)
        chem = (Bm.T @ Bm).reshape(N, N, N, N)          # (pq|rs)
        return np.ascontiguousarray(chem.transpose(0, 2, 1, 3))


def convergent_sigma(o: int, v: int, naux: int | None = None) -> float:
    """sigma_B with naux*v*sigma_B^2 = 3.42 (the o=5, v=19 value of the stated draw)."""
    naux = 3 * (o + v) if naux is None else naux
    return float(np.sqrt(72 * 19 * 0.05**2 / (naux * v)))


def make_workload(o: int, v: int, seed: int = 0, with_amplitudes: bool = False,
                  naux: int | None = None, sigma: float = 0.05) -> Workload:
    rng = np.random.default_rng(seed)
    N = o + v
    naux = 3 * N if naux is None else naux
    e_occ = np.sort(rng.uniform(-1.5, -0.3, o))
    e_vir = np.sort(rng.uniform(0.2, 3.0, v))
    eps = np.concatenate([e_occ, e_vir])
    X = rng.normal(0.0, sigma, (naux, N, N))
    up = np.triu(X)
    B = up + np.transpose(np.triu(X, 1), (0, 2, 1))
    w = Workload(o, v, naux, eps, np.ascontiguousarray(B), sigma=sigma)
    if with_amplitudes:
        x = rng.normal(0.0, 0.01, (o, v))
        y = rng.normal(0.0, 0.01, (o, o, v, v))
        D1 = e_occ[:, None] - e_vir[None, :]
        D2 = D1[:, None, :, None] + D1[None, :, None, :]
        w.t1 = x * np.mean(np.abs(D1)) / np.abs(D1)
        w.t2 = 0.5 * (y + y.transpose(1, 0, 3, 2)) * np.mean(np.abs(D2)) / np.abs(D2)
    return w
