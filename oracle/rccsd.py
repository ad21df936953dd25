"""NumPy float64 restatement of SCESS closed-shell CCSD (``src/Quantum/CC/RCCSD.cpp``).

Test infrastructure only (see the package docstring).  Every function cites the
reference lines it follows.  Tensors use the reference's index meaning:
``eri[p, q, r, s] = <pq|rs> = (pr|qs)`` over spatial MOs, occupied first;
``t1[i, a]``, ``t2[i, j, a, b]`` with ``t2[i,j,a,b] == t2[j,i,b,a]``.
NumPy arrays here are indexed like the reference's Eigen tensors; memory order
is irrelevant to the oracle (the C ABI takes column-major buffers).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_es = lambda spec, *ops: np.einsum(spec, *ops, optimize=True)  # noqa: E731


@dataclass
class RCCSDIntegrals:
    """Integral blocks, RCCSD.cpp:32-44 (chemists' notation blocks named as in PySCF)."""
    ovov: np.ndarray       # (kc|ld) indexed (k,c,l,d)
    oovv: np.ndarray       # (ki|ac) indexed (k,i,a,c)
    ovvo: np.ndarray       # (kc|ai) indexed (k,c,a,i)
    ovvv: np.ndarray       # (kd|ac) indexed (k,d,a,c)
    ovoo: np.ndarray       # (lc|ki) indexed (l,c,k,i)
    oooo_phys: np.ndarray  # <kl|ij> indexed (k,l,i,j)
    vvvv_phys: np.ndarray  # <ab|cd> indexed (a,b,c,d)
    oovv_phys: np.ndarray  # <ij|ab> indexed (i,j,a,b)
    L_oovv_phys: np.ndarray  # 2<ij|ab> - <ij|ba>
    L_ovov: np.ndarray       # 2(kc|ld) - (kd|lc)


def make_integral_blocks(eri: np.ndarray, nocc: int) -> RCCSDIntegrals:
    """``MakeIntegralBlocks``, RCCSD.cpp:47-72."""
    o = nocc
    O, V = slice(0, o), slice(o, None)
    ovov = np.ascontiguousarray(eri[O, O, V, V].transpose(0, 2, 1, 3))   # :55 <kl|cd> -> kcld
    oovv = np.ascontiguousarray(eri[O, V, O, V].transpose(0, 2, 1, 3))   # :57 <ka|ic> -> kiac
    ovvo = np.ascontiguousarray(eri[O, V, V, O].transpose(0, 2, 1, 3))   # :59 <ka|ci> -> kcai
    ovvv = np.ascontiguousarray(eri[O, V, V, V].transpose(0, 2, 1, 3))   # :61 <ka|dc> -> kdac
    ovoo = np.ascontiguousarray(eri[O, O, V, O].transpose(0, 2, 1, 3))   # :63 <lk|ci> -> lcki
    oooo = np.ascontiguousarray(eri[O, O, O, O])                         # :64
    vvvv = np.ascontiguousarray(eri[V, V, V, V])                         # :65
    oovv_phys = np.ascontiguousarray(eri[O, O, V, V])                    # :66
    L_oovv = 2.0 * oovv_phys - oovv_phys.transpose(0, 1, 3, 2)           # :68-69
    L_ovov = 2.0 * ovov - ovov.transpose(0, 3, 2, 1)                     # :70
    return RCCSDIntegrals(ovov, oovv, ovvo, ovvv, ovoo, oooo, vvvv, oovv_phys,
                          np.ascontiguousarray(L_oovv), np.ascontiguousarray(L_ovov))


def plus_transpose(x: np.ndarray) -> np.ndarray:
    """``PlusTranspose``: X_ij^ab + X_ji^ba, RCCSD.cpp:75-77."""
    return x + x.transpose(1, 0, 3, 2)


def make_tau(t1: np.ndarray, t2: np.ndarray) -> np.ndarray:
    """``MakeTau``: tau = t2 + t1 (x) t1, RCCSD.cpp:80-83."""
    return t2 + np.einsum('ia,jb->ijab', t1, t1)


def correlation_energy(ints: RCCSDIntegrals, t1, t2) -> float:
    """``CorrelationEnergy``: sum L_oovv * tau, RCCSD.cpp:85-89."""
    return float(np.sum(ints.L_oovv_phys * make_tau(t1, t2)))


def coupling_energy(f12_energy, t2) -> float:
    """``CouplingEnergy``: sum (2e - e^T) t2, RCCSD.cpp:91-98 (0 without F12)."""
    if f12_energy is None:
        return 0.0
    return float(np.sum((2.0 * f12_energy - f12_energy.transpose(0, 1, 3, 2)) * t2))


def update_amplitudes(ints: RCCSDIntegrals, eia, eijab, t2_driver, t1, t2):
    """One Jacobi update, ``UpdateAmplitudes`` RCCSD.cpp:101-237.

    Returns (t1new / eia, t2new / eijab).  The contraction list, signs and
    grouping follow the reference line by line.
    """
    tau = make_tau(t1, t2)
    Foo = _es('kcld,ilcd->ki', ints.L_ovov, tau)                       # :111
    Fvv = -_es('kcld,klad->ac', ints.L_ovov, tau)                      # :113
    Fov = _es('kcld,ld->kc', ints.L_ovov, t1)                          # :115

    t1new = _es('ac,ic->ia', Fvv, t1)                                  # :119
    t1new -= _es('ki,ka->ia', Foo, t1)                                 # :121
    t1new += 2.0 * _es('kc,kica->ia', Fov, t2)                         # :123
    t1new -= _es('kc,ikca->ia', Fov, t2)                               # :124
    Fov_t1 = _es('kc,ic->ki', Fov, t1)                                 # :127
    t1new += _es('ki,ka->ia', Fov_t1, t1)                              # :128
    t1new += 2.0 * _es('kcai,kc->ia', ints.ovvo, t1)                   # :131
    t1new -= _es('kiac,kc->ia', ints.oovv, t1)                         # :132
    t1new += 2.0 * _es('kdac,ikcd->ia', ints.ovvv, tau)                # :134
    t1new -= _es('kcad,ikcd->ia', ints.ovvv, tau)                      # :135
    t1new -= 2.0 * _es('lcki,klac->ia', ints.ovoo, tau)                # :137
    t1new += _es('kcli,klac->ia', ints.ovoo, tau)                      # :138

    tmp2 = -_es('kibc,ka->abic', ints.oovv, t1)                        # :144
    tmp2 += ints.ovvv.transpose(1, 3, 0, 2)                            # :145 (ia|cb) at (a,b,i,c)
    t2new = plus_transpose(_es('abic,jc->ijab', tmp2, t1))             # :147-148
    tmp2 = _es('kcai,jc->akij', ints.ovvo, t1)                         # :152
    tmp2 += ints.ovoo.transpose(1, 3, 0, 2)                            # :153 (ia|jk) at (a,k,i,j)
    t2new -= plus_transpose(_es('akij,kb->ijab', tmp2, t1))            # :155
    t2new += ints.oovv_phys                                            # :158
    if t2_driver is not None:
        t2new += t2_driver                                             # :159-160

    Loo = Foo + 2.0 * _es('lcki,lc->ki', ints.ovoo, t1)                # :163-164
    Loo -= _es('kcli,lc->ki', ints.ovoo, t1)                           # :165
    Lvv = Fvv + 2.0 * _es('kdac,kd->ac', ints.ovvv, t1)                # :167-168
    Lvv -= _es('kcad,kd->ac', ints.ovvv, t1)                           # :169

    Woooo = ints.oooo_phys.copy()                                      # :172
    Woooo += _es('lcki,jc->klij', ints.ovoo, t1)                       # :173
    Woooo += _es('kclj,ic->klij', ints.ovoo, t1)                       # :174
    Woooo += _es('kcld,ijcd->klij', ints.ovov, tau)                    # :175

    Wvvvv = ints.vvvv_phys.copy()                                      # :178
    Wvvvv -= _es('kdac,kb->abcd', ints.ovvv, t1)                       # :179
    Wvvvv -= _es('kcbd,ka->abcd', ints.ovvv, t1)                       # :180

    Wvoov = ints.ovvo.transpose(2, 0, 3, 1).copy()                     # :183 kcai -> akic
    Wvoov += _es('kcad,id->akic', ints.ovvv, t1)                       # :185
    Wvoov -= _es('kcli,la->akic', ints.ovoo, t1)                       # :186
    Wvoov -= 0.5 * _es('ldkc,ilda->akic', ints.ovov, t2)               # :188-189
    Wvoov -= 0.5 * _es('lckd,ilad->akic', ints.ovov, t2)               # :190-191
    Wvoov += _es('ldkc,ilad->akic', ints.ovov, t2)                     # :192
    tmp = _es('ldkc,id->lkci', ints.ovov, t1)                          # :195
    Wvoov -= _es('lkci,la->akic', tmp, t1)                             # :196

    Wvovo = ints.oovv.transpose(2, 0, 3, 1).copy()                     # :200 kiac -> akci
    Wvovo += _es('kdac,id->akci', ints.ovvv, t1)                       # :202
    Wvovo -= _es('lcki,la->akci', ints.ovoo, t1)                       # :203
    Wvovo -= 0.5 * _es('lckd,ilda->akci', ints.ovov, t2)               # :205-206
    tmp = _es('lckd,id->lcki', ints.ovov, t1)                          # :209
    Wvovo -= _es('lcki,la->akci', tmp, t1)                             # :210

    t2new += _es('klij,klab->ijab', Woooo, tau)                        # :214
    t2new += _es('abcd,ijcd->ijab', Wvvvv, tau)                        # :216
    t2new += plus_transpose(_es('ac,ijcb->ijab', Lvv, t2))             # :218
    t2new -= plus_transpose(_es('ki,kjab->ijab', Loo, t2))             # :220
    tmp = 2.0 * _es('akic,kjcb->ijab', Wvoov, t2)                      # :223-224
    tmp -= _es('akci,kjcb->ijab', Wvovo, t2)                           # :225
    t2new += plus_transpose(tmp)                                       # :226
    tmp = _es('akic,kjbc->ijab', Wvoov, t2)                            # :228
    t2new -= plus_transpose(tmp)                                       # :229
    tmp = _es('bkci,kjac->ijab', Wvovo, t2)                            # :231
    t2new -= plus_transpose(tmp)                                       # :232

    return t1new / eia, t2new / eijab                                  # :235-236


def full_piv_lu_solve(A: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Full-pivoting LU solve with Eigen ``FullPivLU::solve`` semantics.

    The reference solves the bordered DIIS system with ``B.fullPivLu().solve``
    (RCCSD.cpp:268).  Pivots are chosen by largest magnitude over the remaining
    corner; pivots below ``eps * n * |max pivot|`` count as zero, and unknowns
    beyond the numerical rank are set to zero (Eigen's published behaviour).
    The same algorithm runs in the engine's host code.
    """
    A = np.array(A, dtype=np.float64, copy=True)
    n = A.shape[0]
    rowp = np.arange(n)
    colp = np.arange(n)
    nonzero = n
    for k in range(n):
        sub = np.abs(A[k:, k:])
        idx = int(np.argmax(sub))
        i, j = divmod(idx, n - k)
        i += k
        j += k
        if sub.flat[idx] == 0.0:
            nonzero = k
            break
        if i != k:
            A[[k, i], :] = A[[i, k], :]
            rowp[[k, i]] = rowp[[i, k]]
        if j != k:
            A[:, [k, j]] = A[:, [j, k]]
            colp[[k, j]] = colp[[j, k]]
        if k < n - 1:
            A[k + 1:, k] /= A[k, k]
            A[k + 1:, k + 1:] -= np.outer(A[k + 1:, k], A[k, k + 1:])
    diag = np.abs(np.diag(A)[:nonzero])
    maxpiv = diag.max() if nonzero > 0 else 0.0
    thresh = np.finfo(np.float64).eps * n
    rank = int(np.sum(diag > thresh * maxpiv)) if nonzero > 0 else 0
    c = b[rowp].astype(np.float64)
    # forward substitution with unit lower L (all n rows, as Eigen does)
    for i in range(n):
        for j in range(min(i, rank)):
            c[i] -= A[i, j] * c[j]
    y = np.zeros(n)
    for i in range(rank - 1, -1, -1):
        s = c[i]
        for j in range(i + 1, rank):
            s -= A[i, j] * y[j]
        y[i] = s / A[i, i]
    x = np.zeros(n)
    x[colp] = y
    return x


class AmplitudeDIIS:
    """``AmplitudeDIIS``, RCCSD.cpp:240-279."""

    def __init__(self, max_vectors: int):
        self.max_vectors = max_vectors
        self.amplitudes: list[np.ndarray] = []
        self.errors: list[np.ndarray] = []

    def extrapolate(self, amplitudes: np.ndarray, error: np.ndarray) -> np.ndarray:
        self.amplitudes.append(amplitudes)                             # :247-252
        self.errors.append(error)
        if len(self.errors) > self.max_vectors:
            self.amplitudes.pop(0)
            self.errors.pop(0)
        n = len(self.errors)
        B = -np.ones((n + 1, n + 1))                                   # :255-259
        B[n, n] = 0.0
        for i in range(n):
            for j in range(n):
                B[i, j] = float(np.dot(self.errors[i], self.errors[j]))
        maxval = np.abs(B[:n, :n]).max()                               # :262-264
        if maxval > 0.0:
            B[:n, :n] /= maxval
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        coeff = full_piv_lu_solve(B, rhs)                              # :268
        result = np.zeros_like(amplitudes)
        for i in range(n):
            result += coeff[i] * self.amplitudes[i]                    # :270-273
        return result


@dataclass
class RCCSDWfn:
    """``RCCSD_Wfn``, CC.h:105-115 (plus the iteration count and history)."""
    E_CCSD: float = 0.0
    E_F12_Coupling: float = 0.0
    E_T: float = 0.0
    converged: bool = False
    t1: np.ndarray | None = None
    t2: np.ndarray | None = None
    iterations: int = 0
    history: list = field(default_factory=list)


ENERGY_CONVERGENCE = 1.0e-10      # RCCSD.cpp:302
AMPLITUDE_CONVERGENCE = 1.0e-8    # :303
MAX_ITERATIONS = 100              # :304
DIIS_START = 2                    # :306
MAX_DIIS_VECS = 8                 # :307


def denominators(eps: np.ndarray, nocc: int):
    """eia = e_i - e_a and eijab = eia + ejb, RCCSD.cpp:321-331."""
    eia = eps[:nocc, None] - eps[None, nocc:]
    eijab = eia[:, None, :, None] + eia[None, :, None, :]
    return eia, eijab


def solve_rccsd_diis(eri, eps, nocc, f12_residual=None, f12_energy=None,
                     max_iterations=MAX_ITERATIONS, diis_start=DIIS_START,
                     max_diis=MAX_DIIS_VECS, energy_conv=ENERGY_CONVERGENCE,
                     amp_conv=AMPLITUDE_CONVERGENCE, callback=None,
                     t1_init=None, t2_init=None) -> RCCSDWfn:
    """``SolveRCCSD_DIIS``, RCCSD.cpp:295-394.

    ``callback(iteration, E, dE, rms, t1, t2)`` observes every iteration.
    ``t1_init``/``t2_init`` replace the MP2 guess (resume from a checkpoint).
    """
    eri = np.asarray(eri, dtype=np.float64)
    eps = np.asarray(eps, dtype=np.float64)
    ints = make_integral_blocks(eri, nocc)                              # :318
    eia, eijab = denominators(eps, nocc)                               # :321-331
    o, v = eia.shape
    if t1_init is None:
        t1 = np.zeros((o, v))                                          # :334-335
        t2 = ints.oovv_phys.copy()                                     # :336-339
        if f12_residual is not None:
            t2 += f12_residual
        t2 = t2 / eijab
    else:
        t1 = np.array(t1_init, dtype=np.float64)
        t2 = np.array(t2_init, dtype=np.float64)

    diis = AmplitudeDIIS(max_diis)
    E_last = np.finfo(np.float64).max
    wfn = RCCSDWfn()
    for it in range(max_iterations):                                   # :345
        previous = np.concatenate([t1.ravel(order='F'), t2.ravel(order='F')])
        t1, t2 = update_amplitudes(ints, eia, eijab, f12_residual, t1, t2)
        updated = np.concatenate([t1.ravel(order='F'), t2.ravel(order='F')])
        change = updated - previous
        if it >= diis_start:                                           # :354-359
            ext = diis.extrapolate(updated, change)
            t1 = ext[:o * v].reshape((o, v), order='F')
            t2 = ext[o * v:].reshape((o, o, v, v), order='F')
        else:
            diis.extrapolate(updated, change)
        E = correlation_energy(ints, t1, t2) + coupling_energy(f12_energy, t2)   # :361
        dE = abs(E - E_last)
        rms = float(np.linalg.norm(change) / np.sqrt(change.size))     # :363
        E_last = E
        wfn.history.append((it, E, dE, rms))
        if callback is not None:
            callback(it, E, dE, rms, t1, t2)
        wfn.iterations = it + 1
        if dE < energy_conv and rms < amp_conv:                        # :370
            wfn.converged = True
            break
    if not wfn.converged:                                              # :376-380
        return wfn
    wfn.E_CCSD = E_last
    wfn.E_F12_Coupling = coupling_energy(f12_energy, t2)
    wfn.t1 = t1
    wfn.t2 = t2
    return wfn


def ccsd_flops(o: int, v: int) -> float:
    """Algorithmic FLOPs of one ``UpdateAmplitudes`` (contractions a3-a13).

    Summed from the contraction list above, 2*M*N*K per contraction; the
    leading terms are 2o^2v^4 (ladder) + 4ov^4 (Wvvvv dressing) + 16o^3v^3 (rings).
    """
    return float(2 * o**2 * v**4 + 4 * o * v**4 + 16 * o**3 * v**3 + 16 * o**2 * v**3
                 + 4 * o * v**3 + 24 * o**3 * v**2 + 4 * o**4 * v**2 + 4 * o**4 * v)
