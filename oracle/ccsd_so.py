"""Test infrastructure: NumPy float64 restatement of SCESS's spin-orbital
CCSD, CCSD-DIIS and CCSD(T) (``src/Quantum/CC/CCSD.cpp``, ``CCSD-DIIS.cpp``,
``CCSD_T.cpp``) and of the spin integration of the MO integrals
(``src/Quantum/Integrals/IntegralTransforms.cpp:135-162``).  Only the tests
may use it.

In the reference these solvers exist to cross-check the closed-shell ones:
spin-orbital CCSD_DIIS reproduces H2's CCSD energy (``Tests.cpp:550-551``,
1e-6) and H2O/STO-3G's RCCSD energy (``:698-703``, 1e-6), and the
spin-orbital (T) reproduces the closed-shell E_(T) (``:575-577``, 1e-7).  The
tests pin this restatement on the same checks.

Conventions: spin orbital p = 2 x spatial + spin (even alpha, odd beta), as
``TransformFockToMO`` (CCSD.cpp:108-123); occupied spin orbitals first.
``g[p,q,r,s] = <pq||rs>`` over all 2 nmo spin orbitals.
"""
import numpy as np

CC_CONVERGENCE = 1.0e-6      # CCSD.cpp:24, CCSD-DIIS.cpp:20
MAX_ITERATIONS = 50          # CCSD.cpp:26, CCSD-DIIS.cpp:22
MAX_DIIS_VECS = 6            # CCSD-DIIS.cpp:25
DIIS_START = 3               # CCSD-DIIS.cpp:119


def antisymmetrise_spin(mo_chem):
    """AntisymmetriseIntegrateOutSpinClosedShell, IntegralTransforms.cpp:135-162:
    <pq||rs> = (PR|QS) [p~r][q~s] - (PS|QR) [p~s][q~r] (~: same spin)."""
    n = mo_chem.shape[0]
    sp = np.arange(2 * n) // 2
    spin = np.arange(2 * n) % 2
    same = (spin[:, None] == spin[None, :]).astype(np.float64)
    coul = mo_chem[np.ix_(sp, sp, sp, sp)].transpose(0, 2, 1, 3)      # (PR|QS) at [p,q,r,s]
    coul = coul * same[:, None, :, None] * same[None, :, None, :]
    exch = mo_chem[np.ix_(sp, sp, sp, sp)].transpose(0, 2, 3, 1)      # (PS|QR) at [p,q,r,s]
    exch = exch * same[:, None, None, :] * same[None, :, :, None]
    return coul - exch


def spin_eps(eps):
    """Diagonal of the spin-orbital Fock matrix, TransformFockToMO (CCSD.cpp:108-123)."""
    return np.repeat(np.asarray(eps, dtype=np.float64), 2)


def denominators(fe, o):
    """CreateDenominatorTensors, CCSD.cpp:125-148."""
    eo, ev = fe[:o], fe[o:]
    dia = eo[:, None] - ev[None, :]
    dijab = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] \
        - ev[None, None, None, :]
    return dia, dijab


def iterate_ccsd(g, o, dia, dijab, t1, t2):
    """IterateCCSD, CCSD.cpp:161-455 (canonical orbitals: the occupied-virtual
    Fock block the reference adds is zero, TransformFockToMO keeps the diagonal)."""
    O, V = slice(0, o), slice(o, g.shape[0])
    oovv, ovvv, ooov = g[O, O, V, V], g[O, V, V, V], g[O, O, O, V]
    t1t1 = np.einsum('ia,jb->ijab', t1, t1)
    ttau = t2 + 0.5 * t1t1 - 0.5 * t1t1.transpose(0, 1, 3, 2)          # :165-176
    tau = t2 + t1t1 - t1t1.transpose(0, 1, 3, 2)                       # :178-189
    Fae = np.einsum('mf,mafe->ae', t1, ovvv) \
        - 0.5 * np.einsum('mnaf,mnef->ae', ttau, oovv)                 # :191-217
    Fmi = np.einsum('ne,mnie->mi', t1, ooov) \
        + 0.5 * np.einsum('inef,mnef->mi', ttau, oovv)                 # :219-248
    Fme = np.einsum('nf,mnef->me', t1, oovv)                           # :250-261
    P = np.einsum('je,mnie->mnij', t1, ooov)                           # :263-290
    Wmnij = g[O, O, O, O] + P - P.transpose(0, 1, 3, 2) \
        + 0.25 * np.einsum('ijef,mnef->mnij', tau, oovv)
    P = np.einsum('mb,amef->abef', t1, g[V, O, V, V])                  # :292-317
    Wabef = g[V, V, V, V] - P + P.transpose(1, 0, 2, 3) \
        + 0.25 * np.einsum('mnab,mnef->abef', tau, oovv)
    tmp = 0.5 * t2 + t1t1                                              # t1(j,f) t1(n,b) at jnfb, :319-350
    Wmbej = g[O, V, V, O] + np.einsum('jf,mbef->mbej', t1, ovvv) \
        - np.einsum('nb,mnej->mbej', t1, g[O, O, V, O]) \
        - np.einsum('jnfb,mnef->mbej', tmp, oovv)

    r1 = np.einsum('ie,ae->ia', t1, Fae) - np.einsum('ma,mi->ia', t1, Fmi) \
        + np.einsum('imae,me->ia', t2, Fme) - np.einsum('nf,naif->ia', t1, g[O, V, O, V]) \
        - 0.5 * np.einsum('imef,maef->ia', t2, ovvv) \
        - 0.5 * np.einsum('mnae,nmei->ia', t2, g[O, O, V, O])          # :369-402
    r2 = oovv.copy()                                                   # :410-411
    x = Fae - 0.5 * np.einsum('mb,me->be', t1, Fme)                    # :412-421
    P = np.einsum('ijae,be->ijab', t2, x)
    r2 += P - P.transpose(0, 1, 3, 2)
    x = Fmi + 0.5 * np.einsum('me,je->mj', Fme, t1)                    # :423-431
    P = np.einsum('imab,mj->ijab', t2, x)
    r2 += -P + P.transpose(1, 0, 2, 3)
    r2 += 0.5 * np.einsum('mnij,mnab->ijab', Wmnij, tau)               # :433-436
    r2 += 0.5 * np.einsum('ijef,abef->ijab', tau, Wabef)               # :437-440
    P = np.einsum('imae,mbej->ijab', t2, Wmbej) \
        - np.einsum('mbej,ie,ma->ijab', g[O, V, V, O], t1, t1)         # :442-459
    r2 += P - P.transpose(0, 1, 3, 2) - P.transpose(1, 0, 2, 3) + P.transpose(1, 0, 3, 2)
    P = np.einsum('abej,ie->ijab', g[V, V, V, O], t1)                  # :461-468
    r2 += P - P.transpose(1, 0, 2, 3)
    P = np.einsum('mbij,ma->ijab', g[O, V, O, O], t1)                  # :470-476
    r2 += -P + P.transpose(0, 1, 3, 2)
    return r1 / dia, r2 / dijab                                        # :478-479


def energy_ccsd(g, o, t1, t2):
    """CalculateEnergyCCSD, CCSD.cpp:482-509 (the F_ov term is zero)."""
    oovv = g[:o, :o, o:, o:]
    return float(0.25 * np.sum(oovv * t2) + 0.5 * np.einsum('ijab,ia,jb->', oovv, t1, t1))


class SpinCCSDWfn:
    """CCSD_Wfn, CC.h:28-35."""

    def __init__(self):
        self.E_CCSD = 0.0
        self.E_T = 0.0
        self.t1 = None
        self.t2 = None
        self.mints = None
        self.converged = False
        self.iterations = 0
        self.history = []


def ccsd(mo_chem, eps, nocc, diis=True, max_iterations=MAX_ITERATIONS):
    """CCSD (CCSD.cpp:21-106) or, with diis, CCSD_DIIS (CCSD-DIIS.cpp:17-198).
    nocc is the number of doubly occupied spatial orbitals.  Like the
    reference, an unconverged solve returns E_CCSD = 0."""
    g = antisymmetrise_spin(np.asarray(mo_chem, dtype=np.float64))
    o = 2 * int(nocc)
    fe = spin_eps(eps)
    dia, dijab = denominators(fe, o)
    t1 = np.zeros(dia.shape)
    t2 = g[:o, :o, o:, o:] / dijab                                     # CreateInitialT2Tensor :150-157
    amps1, amps2, errs = [], [], []
    E_last, w = np.finfo(np.float64).max, SpinCCSDWfn()
    for it in range(max_iterations):
        if diis:
            amps1.append(t1)
            amps2.append(t2)
        t1, t2 = iterate_ccsd(g, o, dia, dijab, t1, t2)
        if diis:
            errs.append(np.concatenate([(t1 - amps1[-1]).ravel(), (t2 - amps2[-1]).ravel()]))
            amps1[-1], amps2[-1] = t1, t2                              # CCSD-DIIS.cpp:111-115
            if it >= DIIS_START:
                if len(errs) > MAX_DIIS_VECS:
                    del errs[0], amps1[0], amps2[0]
                n = len(errs)
                B = -np.ones((n + 1, n + 1))
                B[n, n] = 0.0
                for i in range(n):
                    for j in range(n):
                        B[i, j] = errs[i] @ errs[j]
                mx = np.max(np.abs(B[:n, :n]))
                if mx > 0.0:
                    B[:n, :n] /= mx
                rhs = np.zeros(n + 1)
                rhs[n] = -1.0
                c = np.linalg.solve(B, rhs)                            # partial-pivot LU
                t1 = sum(c[i] * amps1[i] for i in range(n))
                t2 = sum(c[i] * amps2[i] for i in range(n))
        E = energy_ccsd(g, o, t1, t2)
        w.history.append(E)
        w.iterations = it + 1
        if abs(E - E_last) < CC_CONVERGENCE:
            w.converged = True
            break
        E_last = E
    w.E_CCSD = E if w.converged else 0.0
    w.t1, w.t2, w.mints = t1, t2, g
    return w


def triples_correction(t1, t2, eps, g, o):
    """CalculateTriplesCorrection, CCSD_T.cpp:89-229: connected second-order
    triples, E[4] = 1/4 t2 . (D t3) and E[5] = 1/4 t1 . (g t3); o spin-occupied."""
    O, V = slice(0, o), slice(o, g.shape[0])
    fe = spin_eps(eps)
    eo, ev = fe[:o], fe[o:]
    lhs = np.einsum('dkbc,ijad->ijkabc', g[V, O, V, V], t2, optimize=True)
    t = lhs - lhs.transpose(2, 1, 0, 3, 4, 5) - lhs.transpose(0, 2, 1, 3, 4, 5)  # P(k/ij)
    t = t - t.transpose(0, 1, 2, 4, 3, 5) - t.transpose(0, 1, 2, 5, 4, 3)        # P(a/bc)
    rhs = np.einsum('jklc,ilab->ijkabc', g[O, O, O, V], t2, optimize=True)
    r = rhs - rhs.transpose(1, 0, 2, 3, 4, 5) - rhs.transpose(2, 1, 0, 3, 4, 5)  # P(i/jk)
    r = r - r.transpose(0, 1, 2, 5, 4, 3) - r.transpose(0, 1, 2, 3, 5, 4)        # P(c/ab)
    t = t - r
    d = (eo[:, None, None, None, None, None] + eo[None, :, None, None, None, None]
         + eo[None, None, :, None, None, None] - ev[None, None, None, :, None, None]
         - ev[None, None, None, None, :, None] - ev[None, None, None, None, None, :])
    t = t / d
    x = np.einsum('efbm,ijmaef->ijab', g[V, V, V, O], t, optimize=True)
    vt3 = 0.5 * (x - x.transpose(0, 1, 3, 2))
    x = np.einsum('jemn,imnabe->ijab', g[O, V, O, O], t, optimize=True)
    vt3 -= 0.5 * (x - x.transpose(1, 0, 2, 3))
    e4 = 0.25 * np.sum(t2 * vt3)
    e5 = 0.25 * np.sum(np.einsum('bcjk,ijkabc->ia', g[V, V, O, O], t, optimize=True) * t1)
    return float(e4 + e5)


def ccsd_t(mo_chem, eps, nocc):
    """CCSD_T, CCSD_T.cpp:18-66: CCSD_DIIS, then the triples correction."""
    w = ccsd(mo_chem, eps, nocc, diis=True)
    w.E_T = triples_correction(w.t1, w.t2, eps, w.mints, 2 * int(nocc))
    return w
