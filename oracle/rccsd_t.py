"""NumPy float64 restatement of SCESS closed-shell (T) (``src/Quantum/CC/RCCSD_T.cpp``).

Test infrastructure only.  Two independent forms:

* :func:`rccsd_triples_correction_literal` follows ``RCCSD_TriplesCorrection``
  (RCCSD_T.cpp:17-168) step by step: the P/R/S/Q repack, ``GetW``/``GetV``,
  ``Symmetrise`` over the six simultaneous permutations, r3, the degeneracy
  weight and the final factor 2.  One triple at a time, so only for small v.
* :func:`rccsd_triples_correction` evaluates the same sum with one batch of
  einsums per leading virtual ``a`` (all ``b <= a``, ``c <= b`` at once).  It is
  the cross-check of the literal form and the oracle used at larger sizes.
"""
from __future__ import annotations

import numpy as np


def _repack(eri, nocc, t2):
    """P, R, S, Q of RCCSD_T.cpp:30-56 (index meaning kept, numpy arrays)."""
    o = nocc
    O, V = slice(0, o), slice(o, None)
    # P(i,f,a,b) = (ia|bf) = eri(i, o+b, o+a, o+f)                    :29-41
    P = np.ascontiguousarray(eri[O, V, V, V].transpose(0, 3, 2, 1))
    # R(i,j,m,a) = (ia|mj) = eri(i, m, o+a, j)                          :31-46
    R = np.ascontiguousarray(eri[O, O, V, O].transpose(0, 3, 1, 2))
    # S(i,j,a,b) = (ia|jb) = eri(i, j, o+a, o+b)                        :33-51
    S = np.ascontiguousarray(eri[O, O, V, V])
    # Q(f,j,k,c) = t2(k,j,c,f)                                          :35-56
    Q = np.ascontiguousarray(t2.transpose(3, 1, 0, 2))
    return P, R, S, Q


def rccsd_triples_correction_literal(eri, eps, nocc, t1, t2) -> float:
    """Literal restatement of RCCSD_T.cpp:17-168 (loop over a >= b >= c)."""
    eri = np.asarray(eri, np.float64)
    o = nocc
    v = eri.shape[0] - o
    P, R, S, Q = _repack(eri, o, t2)
    e = np.asarray(eps, np.float64)

    def get_w(a, b, c):
        # w(i,j,k) = sum_f P(i,f,a,b) Q(f,j,k,c) - sum_m R(i,j,m,a) t2(m,k,b,c)   :62-68
        w = np.einsum('if,fjk->ijk', P[:, :, a, b], Q[:, :, :, c])
        w -= np.einsum('ijm,mk->ijk', R[:, :, :, a], t2[:, :, b, c])
        return w

    def get_v(a, b, c):
        # v(i,j,k) = 0.5 t1(k,c) S(i,j,a,b)                                 :70-75
        return 0.5 * S[:, :, a, b][:, :, None] * t1[None, None, :, c]

    def symmetrise(a, b, c, get):
        # X_ijk^abc + X_ikj^acb + X_jik^bac + X_jki^bca + X_kij^cab + X_kji^cba  :78-106
        out = get(a, b, c).copy()
        out += get(a, c, b).transpose(0, 2, 1)        # scratch(i,k,j)
        out += get(b, a, c).transpose(1, 0, 2)        # scratch(j,i,k)
        out += get(b, c, a).transpose(2, 0, 1)        # scratch(j,k,i) at (i,j,k)
        out += get(c, a, b).transpose(1, 2, 0)        # scratch(k,i,j) at (i,j,k)
        out += get(c, b, a).transpose(2, 1, 0)        # scratch(k,j,i)
        return out

    eo = e[:o]
    Dijk = eo[:, None, None] + eo[None, :, None] + eo[None, None, :]
    energy = 0.0
    for a in range(v):                                                  # :111-114
        for b in range(a + 1):
            for c in range(b + 1):
                W = symmetrise(a, b, c, get_w)                          # :131
                Vt = symmetrise(a, b, c, get_v)                         # :132
                deg = 1.0                                               # :135-139
                if a == c:
                    deg = 6.0
                elif a == b or b == c:
                    deg = 2.0
                Y = W + Vt                                              # :145-146
                r3 = (4.0 * Y + Y.transpose(1, 2, 0) + Y.transpose(2, 0, 1)
                      - 2.0 * Y.transpose(2, 1, 0) - 2.0 * Y.transpose(0, 2, 1)
                      - 2.0 * Y.transpose(1, 0, 2))                     # :152-154
                d3 = (Dijk - (e[o + a] + e[o + b] + e[o + c])) * deg    # :147,155
                energy += float(np.sum(W * r3 / d3))                    # :156
    return 2.0 * energy                                                 # :167


def _r3(Y):
    """r3(Y)_ijk = 4Y_ijk + Y_kij + Y_jki - 2Y_kji - 2Y_ikj - 2Y_jik over the last three axes."""
    lead = tuple(range(Y.ndim - 3))
    n = len(lead)

    def tp(p):
        return Y.transpose(lead + tuple(n + x for x in p))
    return (4.0 * Y + tp((1, 2, 0)) + tp((2, 0, 1)) - 2.0 * tp((2, 1, 0))
            - 2.0 * tp((0, 2, 1)) - 2.0 * tp((1, 0, 2)))


def rccsd_triples_correction(eri, eps, nocc, t1, t2, P=None, R=None, S=None) -> float:
    """Vectorised restatement of the same (T) sum, batched over b, c for each a.

    For fixed ``a`` three raw slices are built: A1[b,c] = w^{abc}, A2[b,c] =
    w^{bac}, A3[b,c] = w^{bca} (raw w of RCCSD_T.cpp:62-68); the six permuted
    terms of ``Symmetrise`` are transposes of them.  ``P``, ``R``, ``S`` may be
    given directly (DF inputs) instead of ``eri``.
    """
    o = nocc
    if P is None:
        P, R, S, _ = _repack(np.asarray(eri, np.float64), o, t2)
    v = P.shape[1]
    Q = np.ascontiguousarray(t2.transpose(3, 1, 0, 2))
    e = np.asarray(eps, np.float64)
    eo, ev = e[:o], e[o:]
    Dijk = eo[:, None, None] + eo[None, :, None] + eo[None, None, :]
    energy = 0.0
    for a in range(v):
        n = a + 1
        A1 = np.einsum('ifb,fjkc->bcijk', P[:, :, a, :n], Q[:, :, :, :n], optimize=True)
        A1 -= np.einsum('ijm,mkbc->bcijk', R[:, :, :, a], t2[:, :, :n, :n], optimize=True)
        A2 = np.einsum('ifb,fjkc->bcijk', P[:, :, :n, a], Q[:, :, :, :n], optimize=True)
        A2 -= np.einsum('ijmb,mkc->bcijk', R[:, :, :, :n], t2[:, :, a, :n], optimize=True)
        A3 = np.einsum('ifbc,fjk->bcijk', P[:, :, :n, :n], Q[:, :, :, a], optimize=True)
        A3 -= np.einsum('ijmb,mkc->bcijk', R[:, :, :, :n], t2[:, :, :n, a], optimize=True)
        W = (A1 + A1.transpose(1, 0, 2, 4, 3) + A2.transpose(0, 1, 3, 2, 4)
             + A3.transpose(0, 1, 4, 2, 3) + A2.transpose(1, 0, 3, 4, 2)
             + A3.transpose(1, 0, 4, 3, 2))
        # V_ijk^abc = t1_ia (jb|kc) + t1_jb (ia|kc) + t1_kc (ia|jb)
        Vt = (np.einsum('i,jkbc->bcijk', t1[:, a], S[:, :, :n, :n])
              + np.einsum('jb,ikc->bcijk', t1[:, :n], S[:, :, a, :n])
              + np.einsum('kc,ijb->bcijk', t1[:, :n], S[:, :, a, :n]))
        Y = W + Vt
        r3 = _r3(Y)
        bb, cc = np.meshgrid(np.arange(n), np.arange(n), indexing='ij')
        mask = cc <= bb
        deg = np.ones((n, n))
        deg[(bb == a) | (cc == bb)] = 2.0
        deg[(cc == a)] = 6.0
        dv = ev[a] + ev[:n, None] + ev[None, :n]
        d3 = (Dijk[None, None] - dv[:, :, None, None, None]) * deg[:, :, None, None, None]
        contrib = np.sum(W * r3 / d3, axis=(2, 3, 4))
        energy += float(np.sum(contrib[mask]))
    return 2.0 * energy


def triples_flops(o: int, v: int) -> float:
    """Algorithmic FLOPs of the (T) W build: [v(v+1)(v+2)/6] * 12 o^3 (v+o)."""
    return float(v * (v + 1) * (v + 2) // 6) * 12.0 * o**3 * (v + o)
