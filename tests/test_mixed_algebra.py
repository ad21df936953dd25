"""The algebra behind the mixed form's residual, checked on the CPU against the
FP64 oracle (a NumPy transcription with the einsum specs of rccsd.cu):

* the reassociated contraction list (T1 dressing of Wvvvv folded into the
  ladder, the :144-147 term reassociated) computes UpdateAmplitudes'
  numerators (RCCSD.cpp:101-237);
* the change of the residual as rccsd_residual_delta expands it (every product
  A1 B1 - A0 B0 = dA B1 + A0 dB, the constant terms dropped) gives
  R(T0 + d) = R(T0) + dR exactly;
* the particle ladder in its symmetric / antisymmetric form (ladder_pm: pairs
  c <= d and c < d, results over pairs i <= j, a <= b) equals the plain
  contraction sum_cd <ab|cd> tau(i,j,c,d).
"""
import numpy as np

import oracle
from scess_gb300.synthetic import convergent_sigma, make_workload


def es(spec, a, b):
    return np.einsum(spec, a, b, optimize=True)


def forward(I, t1, t2, o, v):
    """rccsd_residual's reassociated list; returns R1, R2 and its intermediates."""
    w = {}
    tau = t2 + np.einsum('ia,jb->ijab', t1, t1)
    w['tau'] = tau
    w['Foo'] = es('kcld,ilcd->ki', I.L_ovov, tau)
    w['Fvv'] = -es('kcld,klad->ac', I.L_ovov, tau)
    w['Fov'] = es('kcld,ld->kc', I.L_ovov, t1)
    R1 = es('ac,ic->ia', w['Fvv'], t1) - es('ki,ka->ia', w['Foo'], t1)
    R1 += 2 * es('kc,kica->ia', w['Fov'], t2) - es('kc,ikca->ia', w['Fov'], t2)
    w['Fovt1'] = es('kc,ic->ki', w['Fov'], t1)
    R1 += es('ki,ka->ia', w['Fovt1'], t1)
    R1 += 2 * es('kcai,kc->ia', I.ovvo, t1) - es('kiac,kc->ia', I.oovv, t1)
    R1 += 2 * es('kdac,ikcd->ia', I.ovvv, tau) - es('kcad,ikcd->ia', I.ovvv, tau)
    R1 += -2 * es('lcki,klac->ia', I.ovoo, tau) + es('kcli,klac->ia', I.ovoo, tau)
    w['tmp_kibj'] = es('kibc,jc->kibj', I.oovv, t1)
    X = es('iacb,jc->ijab', I.ovvv, t1) - es('kibj,ka->ijab', w['tmp_kibj'], t1)
    w['tmp_akij'] = es('kcai,jc->akij', I.ovvo, t1) + np.einsum('iajk->akij', I.ovoo)
    X -= es('akij,kb->ijab', w['tmp_akij'], t1)
    R2 = I.oovv_phys.copy()
    w['Loo'] = w['Foo'] + 2 * es('lcki,lc->ki', I.ovoo, t1) - es('kcli,lc->ki', I.ovoo, t1)
    w['Lvv'] = w['Fvv'] + 2 * es('kdac,kd->ac', I.ovvv, t1) - es('kcad,kd->ac', I.ovvv, t1)
    w['Woooo'] = (I.oooo_phys + es('lcki,jc->klij', I.ovoo, t1) + es('kclj,ic->klij', I.ovoo, t1)
                  + es('kcld,ijcd->klij', I.ovov, tau))
    W = (np.einsum('kcai->akic', I.ovvo) + es('kcad,id->akic', I.ovvv, t1)
         - es('kcli,la->akic', I.ovoo, t1))
    W += (-0.5 * es('ldkc,ilda->akic', I.ovov, t2) - 0.5 * es('lckd,ilad->akic', I.ovov, t2)
          + es('ldkc,ilad->akic', I.ovov, t2))
    w['tmp_lkci'] = es('ldkc,id->lkci', I.ovov, t1)
    W -= es('lkci,la->akic', w['tmp_lkci'], t1)
    w['Wvoov'] = W
    W = (np.einsum('kiac->akci', I.oovv) + es('kdac,id->akci', I.ovvv, t1)
         - es('lcki,la->akci', I.ovoo, t1) - 0.5 * es('lckd,ilda->akci', I.ovov, t2))
    w['tmp_lcki'] = es('lckd,id->lcki', I.ovov, t1)
    W -= es('lcki,la->akci', w['tmp_lcki'], t1)
    w['Wvovo'] = W
    R2 += es('klij,klab->ijab', w['Woooo'], tau)
    R2 += es('abcd,ijcd->ijab', I.vvvv_phys, tau)
    w['Yd'] = es('kcbd,ijcd->kbij', I.ovvv, tau)
    X -= es('ka,kbij->ijab', t1, w['Yd'])
    X += es('ac,ijcb->ijab', w['Lvv'], t2) - es('ki,kjab->ijab', w['Loo'], t2)
    X += 2 * es('akic,kjcb->ijab', w['Wvoov'], t2) - es('akci,kjcb->ijab', w['Wvovo'], t2)
    X -= es('akic,kjbc->ijab', w['Wvoov'], t2) + es('bkci,kjac->ijab', w['Wvovo'], t2)
    R2 += X + X.transpose(1, 0, 3, 2)
    return R1, R2, w


def delta(I, t1_0, t1_1, t2_1, dt1, dt2, w0):
    """rccsd_residual_delta: dR = R(T0 + d) - R(T0) from the base intermediates w0."""
    def E2(spec, dA, B1, A0, dB):
        return es(spec, dA, B1) + es(spec, A0, dB)
    w = {}
    dtau = dt2 + np.einsum('ia,jb->ijab', dt1, t1_1) + np.einsum('ia,jb->ijab', t1_0, dt1)
    tau_1 = w0['tau'] + dtau
    w['Foo'] = es('kcld,ilcd->ki', I.L_ovov, dtau)
    w['Fvv'] = -es('kcld,klad->ac', I.L_ovov, dtau)
    w['Fov'] = es('kcld,ld->kc', I.L_ovov, dt1)
    R1 = E2('ac,ic->ia', w['Fvv'], t1_1, w0['Fvv'], dt1) - E2('ki,ka->ia', w['Foo'], t1_1, w0['Foo'], dt1)
    R1 += 2 * E2('kc,kica->ia', w['Fov'], t2_1, w0['Fov'], dt2)
    R1 -= E2('kc,ikca->ia', w['Fov'], t2_1, w0['Fov'], dt2)
    w['Fovt1'] = E2('kc,ic->ki', w['Fov'], t1_1, w0['Fov'], dt1)
    R1 += E2('ki,ka->ia', w['Fovt1'], t1_1, w0['Fovt1'], dt1)
    R1 += 2 * es('kcai,kc->ia', I.ovvo, dt1) - es('kiac,kc->ia', I.oovv, dt1)
    R1 += 2 * es('kdac,ikcd->ia', I.ovvv, dtau) - es('kcad,ikcd->ia', I.ovvv, dtau)
    R1 += -2 * es('lcki,klac->ia', I.ovoo, dtau) + es('kcli,klac->ia', I.ovoo, dtau)
    w['tmp_kibj'] = es('kibc,jc->kibj', I.oovv, dt1)
    X = es('iacb,jc->ijab', I.ovvv, dt1) - E2('kibj,ka->ijab', w['tmp_kibj'], t1_1, w0['tmp_kibj'], dt1)
    w['tmp_akij'] = es('kcai,jc->akij', I.ovvo, dt1)
    X -= E2('akij,kb->ijab', w['tmp_akij'], t1_1, w0['tmp_akij'], dt1)
    w['Loo'] = w['Foo'] + 2 * es('lcki,lc->ki', I.ovoo, dt1) - es('kcli,lc->ki', I.ovoo, dt1)
    w['Lvv'] = w['Fvv'] + 2 * es('kdac,kd->ac', I.ovvv, dt1) - es('kcad,kd->ac', I.ovvv, dt1)
    w['Woooo'] = (es('lcki,jc->klij', I.ovoo, dt1) + es('kclj,ic->klij', I.ovoo, dt1)
                  + es('kcld,ijcd->klij', I.ovov, dtau))
    W = es('kcad,id->akic', I.ovvv, dt1) - es('kcli,la->akic', I.ovoo, dt1)
    W += (-0.5 * es('ldkc,ilda->akic', I.ovov, dt2) - 0.5 * es('lckd,ilad->akic', I.ovov, dt2)
          + es('ldkc,ilad->akic', I.ovov, dt2))
    w['tmp_lkci'] = es('ldkc,id->lkci', I.ovov, dt1)
    W -= E2('lkci,la->akic', w['tmp_lkci'], t1_1, w0['tmp_lkci'], dt1)
    w['Wvoov'] = W
    W = (es('kdac,id->akci', I.ovvv, dt1) - es('lcki,la->akci', I.ovoo, dt1)
         - 0.5 * es('lckd,ilda->akci', I.ovov, dt2))
    w['tmp_lcki'] = es('lckd,id->lcki', I.ovov, dt1)
    W -= E2('lcki,la->akci', w['tmp_lcki'], t1_1, w0['tmp_lcki'], dt1)
    w['Wvovo'] = W
    R2 = E2('klij,klab->ijab', w['Woooo'], tau_1, w0['Woooo'], dtau)
    R2 += es('abcd,ijcd->ijab', I.vvvv_phys, dtau)
    w['Yd'] = es('kcbd,ijcd->kbij', I.ovvv, dtau)
    X -= es('ka,kbij->ijab', dt1, w0['Yd']) + es('ka,kbij->ijab', t1_1, w['Yd'])
    X += E2('ac,ijcb->ijab', w['Lvv'], t2_1, w0['Lvv'], dt2)
    X -= E2('ki,kjab->ijab', w['Loo'], t2_1, w0['Loo'], dt2)
    X += 2 * E2('akic,kjcb->ijab', w['Wvoov'], t2_1, w0['Wvoov'], dt2)
    X -= E2('akci,kjcb->ijab', w['Wvovo'], t2_1, w0['Wvovo'], dt2)
    X -= E2('akic,kjbc->ijab', w['Wvoov'], t2_1, w0['Wvoov'], dt2)
    X -= E2('bkci,kjac->ijab', w['Wvovo'], t2_1, w0['Wvovo'], dt2)
    R2 += X + X.transpose(1, 0, 3, 2)
    return R1, R2


def ladder_pm(V, tau):
    """ladder_pm / ladder_unpack: sum_cd V(a,b,c,d) tau(i,j,c,d) over pairs."""
    o, v = tau.shape[0], V.shape[0]
    pu = lambda n: [(p, q) for q in range(n) for p in range(q + 1)]  # noqa: E731
    ps = lambda n: [(p, q) for q in range(n) for p in range(q)]  # noqa: E731
    Vp = np.array([[V[a, b, c, d] + V[a, b, d, c] if c < d else V[a, b, c, c] for c, d in pu(v)]
                   for a, b in pu(v)])
    Vm = np.array([[V[a, b, c, d] - V[a, b, d, c] for c, d in ps(v)] for a, b in ps(v)])
    Tp = np.array([[0.5 * (tau[i, j, c, d] + tau[i, j, d, c]) for c, d in pu(v)] for i, j in pu(o)])
    Tm = np.array([[0.5 * (tau[i, j, c, d] - tau[i, j, d, c]) for c, d in ps(v)] for i, j in ps(o)])
    Sp, Sm = Tp @ Vp.T, Tm @ Vm.T
    out = np.zeros((o, o, v, v))
    for i in range(o):
        for j in range(o):
            for a in range(v):
                for b in range(v):
                    i0, j0, a0, b0 = min(i, j), max(i, j), min(a, b), max(a, b)
                    s = Sp[j0 * (j0 + 1) // 2 + i0, b0 * (b0 + 1) // 2 + a0]
                    if i != j and a != b:
                        m = Sm[j0 * (j0 - 1) // 2 + i0, b0 * (b0 - 1) // 2 + a0]
                        s += m if (i < j) == (a < b) else -m
                    out[i, j, a, b] = s
    return out


def _case(o=4, v=11, seed=2):
    w = make_workload(o, v, seed=1, sigma=convergent_sigma(o, v))
    I = oracle.make_integral_blocks(w.eri(), o)
    eia, eijab = oracle.rccsd.denominators(w.eps, o)
    rng = np.random.default_rng(seed)
    sym = lambda x: 0.5 * (x + x.transpose(1, 0, 3, 2))  # noqa: E731
    t1 = 0.02 * rng.standard_normal((o, v))
    t2 = sym(0.02 * rng.standard_normal((o, o, v, v)))
    d1 = 1e-3 * rng.standard_normal((o, v))
    d2 = sym(1e-3 * rng.standard_normal((o, o, v, v)))
    return w, I, eia, eijab, t1, t2, d1, d2


def _rel(x, ref):
    return float(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))


def test_reassociated_list_is_update_amplitudes():
    w, I, eia, eijab, t1, t2, _, _ = _case()
    R1, R2, _ = forward(I, t1, t2, w.o, w.v)
    u1, u2 = oracle.update_amplitudes(I, eia, eijab, None, t1, t2)
    assert _rel(R1 / eia, u1) < 1e-14 and _rel(R2 / eijab, u2) < 1e-14


def test_delta_expansion_is_exact():
    w, I, eia, eijab, t1, t2, d1, d2 = _case()
    R1, R2, w0 = forward(I, t1, t2, w.o, w.v)
    dR1, dR2 = delta(I, t1, t1 + d1, t2 + d2, d1, d2, w0)
    v1, v2 = oracle.update_amplitudes(I, eia, eijab, None, t1 + d1, t2 + d2)
    assert _rel((R1 + dR1) / eia, v1) < 1e-14
    assert _rel((R2 + dR2) / eijab, v2) < 1e-14


def test_symmetric_antisymmetric_ladder():
    rng = np.random.default_rng(0)
    o, v = 4, 7
    Vf = rng.standard_normal((v, v, v, v))
    V = 0.5 * (Vf + Vf.transpose(1, 0, 3, 2))            # <ab|cd> = <ba|dc>
    y = rng.standard_normal((o, o, v, v))
    tau = 0.5 * (y + y.transpose(1, 0, 3, 2))           # tau(ijcd) = tau(jidc)
    assert _rel(ladder_pm(V, tau), np.einsum('abcd,ijcd->ijab', V, tau)) < 1e-14
