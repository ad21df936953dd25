"""CPU tests of the CCSD-F12b coupling restatement (CCSD_F12b.cpp:31-35, 83-91)."""
import numpy as np

import oracle


def _tensors(N, o, seed):
    rng = np.random.default_rng(seed)
    eri = rng.standard_normal((N, N, N, N))
    f12 = rng.standard_normal((N, N, N, N))
    rep = rng.standard_normal((N, N, N, N))
    C = rng.standard_normal((o, o, N - o, N - o))
    return eri, f12, rep, C


def test_fixed_amplitudes_are_the_sp_geminal_contraction():
    """3/8 X_ij + 1/8 X_ji equals sum_kl c_ij^kl X_kl with c_ij^kl =
    3/8 d_ik d_jl + 1/8 d_il d_jk, written out."""
    o, v = 3, 4
    X = np.random.default_rng(0).standard_normal((o, o, v, v))
    d = np.eye(o)
    c = 0.375 * np.einsum('ik,jl->ijkl', d, d) + 0.125 * np.einsum('il,jk->ijkl', d, d)
    assert np.allclose(oracle.contract_fixed_amplitudes(X), np.einsum('ijkl,klab->ijab', c, X))


def test_coupling_by_loops():
    N, o = 5, 2
    eri, f12, rep, C = _tensors(N, o, 1)
    res, en = oracle.f12b_coupling(eri, f12, rep, C, o)
    v = N - o
    V = np.zeros((o, o, v, v))
    for k in range(o):
        for l in range(o):
            for a in range(v):
                for b in range(v):
                    V[k, l, a, b] = rep[k, l, o + a, o + b] - sum(
                        eri[o + a, o + b, r, s] * f12[k, l, r, s] for r in range(N) for s in range(N))
    X = C + V
    assert np.allclose(res, 0.375 * X + 0.125 * X.transpose(1, 0, 2, 3))
    assert np.allclose(en, 0.375 * C + 0.125 * C.transpose(1, 0, 2, 3))
