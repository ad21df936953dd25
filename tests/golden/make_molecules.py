"""Generate the real-molecule golden fixtures (MO integrals + orbital energies).

The reference's regression pins (``src/SCESS/Tests.cpp:34-75``) are energies
of H2/STO-3G, H2O/STO-3G and H2O/cc-pVDZ.  The reference's own integral stack
(Libint2) cannot be built here, so this script computes the integrals from the
McMurchie-Davidson Hermite-Gaussian formulas, runs a closed-shell RHF (DIIS,
1e-12), and writes the MO-basis physicists' integrals ``eri[p,q,r,s] =
<pq|rs>`` (occupied first) with the orbital energies, plus the AO integrals
and the MO coefficients they were transformed with (inputs of the AO->MO
transform test).  The tests then check the
oracle's CCSD/(T) energies on these inputs against the pins, and the CUDA
engine against the oracle.

* Basis sets: the reference's Basis Set Exchange JSON files
  (``Assets/Basis/Pople/STO-3G.json``, ``Assets/Basis/Dunning/cc-pVDZ.json``),
  read at generation time; cc-pVDZ d shells are solid harmonic
  (``function_type: gto_spherical``).
* Geometries: ``Molecule::GenerateWaterMolecule`` / ``GenerateHydrogenMolecule``
  (``src/Quantum/Molecule.cpp:194-216``), converted with PySCF's Bohr radius
  0.52917721092 A because the pins were produced by PySCF from those angstrom
  coordinates (``Scripts/verification/spherical_check.py``).
* Boys function: ``F_n(T) = Gamma(n+1/2) P(n+1/2, T) / (2 T^(n+1/2))`` with
  the regularised lower incomplete gamma from SciPy (series limit 1/(2n+1) at 0).

Run: ``python tests/golden/make_molecules.py /path/to/SCESS`` (writes
``tests/golden/<name>.npz``).  Only the unique 8-fold-symmetric integrals
are stored; :func:`load` in ``tests/golden/__init__.py`` expands them.
"""
from __future__ import annotations

import itertools
import json
import os
import sys

import numpy as np
from scipy.special import gamma, gammainc

BOHR = 0.52917721092
ZNUC = {'H': 1.0, 'O': 8.0}
ZSYM = {'H': '1', 'O': '8'}


def boys(nmax: int, T: np.ndarray) -> np.ndarray:
    """F_n(T) for n = 0..nmax, shape (nmax+1,) + T.shape."""
    T = np.asarray(T, dtype=np.float64)
    out = np.empty((nmax + 1,) + T.shape)
    small = T < 1e-13
    Ts = np.where(small, 1.0, T)
    for n in range(nmax + 1):
        a = n + 0.5
        val = gamma(a) * gammainc(a, Ts) / (2.0 * Ts ** a)
        out[n] = np.where(small, 1.0 / (2 * n + 1) - T / (2 * n + 3), val)
    return out


def cart_components(l: int):
    return [(lx, ly, l - lx - ly) for lx in range(l, -1, -1) for ly in range(l - lx, -1, -1)]


def sph_transform(l: int) -> np.ndarray:
    """Rows: real solid harmonics as combinations of Cartesian components (any basis of the span)."""
    if l < 2:
        return np.eye(len(cart_components(l)))
    assert l == 2
    comps = cart_components(2)    # xx, xy, xz, yy, yz, zz
    idx = {c: i for i, c in enumerate(comps)}
    T = np.zeros((5, 6))
    T[0, idx[(1, 1, 0)]] = 1.0                                  # xy
    T[1, idx[(0, 1, 1)]] = 1.0                                  # yz
    T[2, idx[(0, 0, 2)]] = 2.0                                  # 2zz - xx - yy
    T[2, idx[(2, 0, 0)]] = -1.0
    T[2, idx[(0, 2, 0)]] = -1.0
    T[3, idx[(1, 0, 1)]] = 1.0                                  # xz
    T[4, idx[(2, 0, 0)]] = 1.0                                  # xx - yy
    T[4, idx[(0, 2, 0)]] = -1.0
    return T


class Shell:
    def __init__(self, center, l, exps, coefs, spherical):
        self.center = np.asarray(center, float)
        self.l = l
        self.exps = np.asarray(exps, float)
        # primitive normalisation of the axial component x^l
        norm = (2 * self.exps / np.pi) ** 0.75 * (4 * self.exps) ** (l / 2.0)
        dfac = np.prod([np.prod(np.arange(2 * l - 1, 0, -2)) if l > 0 else 1.0])
        self.coefs = np.asarray(coefs, float) * norm / np.sqrt(dfac)
        self.comps = cart_components(l)
        self.spherical = spherical and l >= 2


def load_basis(path: str, atoms):
    data = json.load(open(path))
    shells = []
    for sym, xyz in atoms:
        el = data['elements'][ZSYM[sym]]
        for sh in el['electron_shells']:
            exps = [float(e) for e in sh['exponents']]
            ams = sh['angular_momentum']
            sph = sh['function_type'] == 'gto_spherical'
            for j, cs in enumerate(sh['coefficients']):
                l = ams[j] if len(ams) > 1 else ams[0]
                prims = [(e, float(c)) for e, c in zip(exps, cs) if float(c) != 0.0]
                shells.append(Shell(xyz, l, [p[0] for p in prims], [p[1] for p in prims], sph))
    return shells


def hermite_E(la, lb, Ax, Bx, a, b):
    """E[i][j][t] arrays (broadcast over primitive exponents a[:,None], b[None,:])."""
    p = a + b
    q = a * b / p
    Qx = Ax - Bx
    E = {}
    E[(0, 0, 0)] = np.exp(-q * Qx * Qx)

    def get(i, j, t):
        if t < 0 or t > i + j or i < 0 or j < 0:
            return 0.0
        key = (i, j, t)
        if key in E:
            return E[key]
        if i > 0:
            val = (get(i - 1, j, t - 1) / (2 * p) - (q * Qx / a) * get(i - 1, j, t)
                   + (t + 1) * get(i - 1, j, t + 1))
        else:
            val = (get(i, j - 1, t - 1) / (2 * p) + (q * Qx / b) * get(i, j - 1, t)
                   + (t + 1) * get(i, j - 1, t + 1))
        E[key] = val
        return val
    return get


def hermite_R(L, alpha, PCx, PCy, PCz):
    """R_{tuv}(alpha, PC) for t+u+v <= L as a dict."""
    T = alpha * (PCx ** 2 + PCy ** 2 + PCz ** 2)
    F = boys(L, T)
    memo = {}

    def R(n, t, u, v):
        if t < 0 or u < 0 or v < 0:
            return 0.0
        key = (n, t, u, v)
        if key in memo:
            return memo[key]
        if t == u == v == 0:
            val = (-2 * alpha) ** n * F[n]
        elif t > 0:
            val = (t - 1) * R(n + 1, t - 2, u, v) + PCx * R(n + 1, t - 1, u, v)
        elif u > 0:
            val = (u - 1) * R(n + 1, t, u - 2, v) + PCy * R(n + 1, t, u - 1, v)
        else:
            val = (v - 1) * R(n + 1, t, u, v - 2) + PCz * R(n + 1, t, u, v - 1)
        memo[key] = val
        return val
    return {(t, u, v): R(0, t, u, v) for t in range(L + 1) for u in range(L + 1 - t)
            for v in range(L + 1 - t - u)}


class Pair:
    """Primitive-pair Hermite data for a shell pair."""

    def __init__(self, sa: Shell, sb: Shell):
        a = sa.exps[:, None]
        b = sb.exps[None, :]
        self.p = a + b
        self.P = (a[..., None] * sa.center + b[..., None] * sb.center) / self.p[..., None]
        self.cc = sa.coefs[:, None] * sb.coefs[None, :]
        Ex = hermite_E(sa.l, sb.l, sa.center[0], sb.center[0], a, b)
        Ey = hermite_E(sa.l, sb.l, sa.center[1], sb.center[1], a, b)
        Ez = hermite_E(sa.l, sb.l, sa.center[2], sb.center[2], a, b)
        L = sa.l + sb.l
        self.herm = [(t, u, v) for t in range(L + 1) for u in range(L + 1 - t) for v in range(L + 1 - t - u)]
        na, nb = len(sa.comps), len(sb.comps)
        shp = self.p.shape
        self.E = np.zeros((na, nb, len(self.herm)) + shp)
        for i, ca in enumerate(sa.comps):
            for j, cb in enumerate(sb.comps):
                for h, (t, u, v) in enumerate(self.herm):
                    self.E[i, j, h] = (np.broadcast_to(Ex(ca[0], cb[0], t), shp)
                                       * Ey(ca[1], cb[1], u) * Ez(ca[2], cb[2], v))
        self.Ex, self.Ey, self.Ez = Ex, Ey, Ez
        self.sa, self.sb = sa, sb


def one_electron(shells, atoms):
    nbf = sum(len(s.comps) for s in shells)
    S = np.zeros((nbf, nbf))
    Tk = np.zeros((nbf, nbf))
    Vn = np.zeros((nbf, nbf))
    offs = np.cumsum([0] + [len(s.comps) for s in shells])
    for ia, sa in enumerate(shells):
        for ib, sb in enumerate(shells):
            pr = Pair(sa, sb)
            p = pr.p
            a = sa.exps[:, None]
            b = sb.exps[None, :]
            pref = (np.pi / p) ** 1.5 * pr.cc
            for i, ca in enumerate(sa.comps):
                for j, cb in enumerate(sb.comps):
                    def ov(dx, dy, dz, ca=ca, cb=cb):
                        lb = (cb[0] + dx, cb[1] + dy, cb[2] + dz)
                        if min(lb) < 0:
                            return 0.0
                        return (pr.Ex(ca[0], lb[0], 0) * pr.Ey(ca[1], lb[1], 0) * pr.Ez(ca[2], lb[2], 0))
                    s = ov(0, 0, 0)
                    S[offs[ia] + i, offs[ib] + j] = np.sum(pref * s)
                    # kinetic: -1/2 <a|nabla^2|b> via Obara-Saika-style shifts of b
                    kin = 0.0
                    for d, (dx, dy, dz) in enumerate([(1, 0, 0), (0, 1, 0), (0, 0, 1)]):
                        lbd = cb[d]
                        term = (b * (2 * lbd + 1) * s - 2 * b * b * ov(2 * dx, 2 * dy, 2 * dz)
                                - 0.5 * lbd * (lbd - 1) * ov(-2 * dx, -2 * dy, -2 * dz))
                        kin = kin + term
                    Tk[offs[ia] + i, offs[ib] + j] = np.sum(pref * kin)
            for sym, C in atoms:
                PC = pr.P - C
                R = hermite_R(sa.l + sb.l, p, PC[..., 0], PC[..., 1], PC[..., 2])
                for i in range(len(sa.comps)):
                    for j in range(len(sb.comps)):
                        acc = 0.0
                        for h, tuv in enumerate(pr.herm):
                            acc = acc + pr.E[i, j, h] * R[tuv]
                        Vn[offs[ia] + i, offs[ib] + j] += -ZNUC[sym] * np.sum(2 * np.pi / p * pr.cc * acc)
    return S, Tk, Vn


def two_electron(shells):
    nbf = sum(len(s.comps) for s in shells)
    offs = np.cumsum([0] + [len(s.comps) for s in shells])
    eri = np.zeros((nbf, nbf, nbf, nbf))
    ns = len(shells)
    pairs = {}
    for i in range(ns):
        for j in range(i + 1):
            pairs[(i, j)] = Pair(shells[i], shells[j])
    keys = list(pairs.keys())
    for x, kab in enumerate(keys):
        pab = pairs[kab]
        for kcd in keys[:x + 1]:
            pcd = pairs[kcd]
            p = pab.p[:, :, None, None]
            q = pcd.p[None, None, :, :]
            alpha = p * q / (p + q)
            PQ = pab.P[:, :, None, None, :] - pcd.P[None, None, :, :, :]
            L = pab.sa.l + pab.sb.l + pcd.sa.l + pcd.sb.l
            R = hermite_R(L, alpha, PQ[..., 0], PQ[..., 1], PQ[..., 2])
            pref = 2 * np.pi ** 2.5 / (p * q * np.sqrt(p + q))
            pref = pref * pab.cc[:, :, None, None] * pcd.cc[None, None, :, :]
            nh1, nh2 = len(pab.herm), len(pcd.herm)
            Rm = np.empty((nh1, nh2) + alpha.shape)
            for h1, (t, u, v) in enumerate(pab.herm):
                for h2, (tt, uu, vv) in enumerate(pcd.herm):
                    Rm[h1, h2] = R[(t + tt, u + uu, v + vv)] * (-1) ** (tt + uu + vv)
            block = np.einsum('ijhab,klgcd,hgabcd,abcd->ijkl', pab.E, pcd.E, Rm, pref, optimize=True)
            ia, ib = kab
            ic, id_ = kcd
            sl = lambda s: slice(offs[s], offs[s + 1])  # noqa: E731
            for perm_ab in [(ia, ib, block), (ib, ia, block.transpose(1, 0, 2, 3))]:
                a_, b_, bl = perm_ab
                for perm_cd in [(ic, id_, bl), (id_, ic, bl.transpose(0, 1, 3, 2))]:
                    c_, d_, bl2 = perm_cd
                    eri[sl(a_), sl(b_), sl(c_), sl(d_)] = bl2
                    eri[sl(c_), sl(d_), sl(a_), sl(b_)] = bl2.transpose(2, 3, 0, 1)
    return eri


def cart_to_sph(shells):
    blocks = []
    for s in shells:
        blocks.append(sph_transform(s.l) if s.spherical else np.eye(len(s.comps)))
    nrow = sum(b.shape[0] for b in blocks)
    ncol = sum(b.shape[1] for b in blocks)
    T = np.zeros((nrow, ncol))
    r = c = 0
    for b in blocks:
        T[r:r + b.shape[0], c:c + b.shape[1]] = b
        r += b.shape[0]
        c += b.shape[1]
    return T


def rhf(S, H, eri, nocc, enuc, conv=1e-12, maxit=200):
    """Closed-shell RHF with Pulay DIIS; returns (E, eps, C)."""
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    e, Cp = np.linalg.eigh(X.T @ H @ X)
    C = X @ Cp
    D = C[:, :nocc] @ C[:, :nocc].T
    focks, errs = [], []
    E_old = 0.0
    for it in range(maxit):
        J = np.einsum('pqrs,rs->pq', eri, D)
        K = np.einsum('prqs,rs->pq', eri, D)
        F = H + 2 * J - K
        E = np.sum(D * (H + F)) + enuc
        err = F @ D @ S - S @ D @ F
        focks.append(F)
        errs.append(err)
        if len(focks) > 8:
            focks.pop(0)
            errs.pop(0)
        n = len(focks)
        Bm = -np.ones((n + 1, n + 1))
        Bm[n, n] = 0
        for i in range(n):
            for j in range(n):
                Bm[i, j] = np.sum(errs[i] * errs[j])
        rhs = np.zeros(n + 1)
        rhs[n] = -1
        cvec = np.linalg.lstsq(Bm, rhs, rcond=None)[0]
        Fd = sum(cvec[i] * focks[i] for i in range(n))
        e, Cp = np.linalg.eigh(X.T @ Fd @ X)
        C = X @ Cp
        D = C[:, :nocc] @ C[:, :nocc].T
        if abs(E - E_old) < conv and np.abs(err).max() < 1e-9:
            break
        E_old = E
    J = np.einsum('pqrs,rs->pq', eri, D)
    K = np.einsum('prqs,rs->pq', eri, D)
    F = H + 2 * J - K
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    C = X @ Cp
    D = C[:, :nocc] @ C[:, :nocc].T
    E = np.sum(D * (H + H + 2 * J - K)) + enuc
    return E, e, C


def molecule(name):
    if name == 'h2':
        d = 0.7122300374 / BOHR
        return [('H', np.array([0.0, 0.0, 0.0])), ('H', np.array([d, 0.0, 0.0]))]
    return [('H', np.array([0.7569520, -0.586349, 0.0]) / BOHR), ('O', np.zeros(3)),
            ('H', np.array([-0.7569520, -0.586349, 0.0]) / BOHR)]


def compute(name, basis_path, nocc):
    atoms = molecule(name)
    shells = load_basis(basis_path, atoms)
    S, Tk, Vn = one_electron(shells, atoms)
    eri_c = two_electron(shells)
    T = cart_to_sph(shells)
    S = T @ S @ T.T
    H = T @ (Tk + Vn) @ T.T
    eri = np.einsum('pi,qj,ijkl,rk,sl->pqrs', T, T, eri_c, T, T, optimize=True)
    nrm = 1.0 / np.sqrt(np.diag(S))
    S = S * np.outer(nrm, nrm)
    H = H * np.outer(nrm, nrm)
    eri = eri * nrm[:, None, None, None] * nrm[None, :, None, None] * nrm[None, None, :, None] * nrm[None, None, None, :]
    enuc = 0.0
    for (s1, c1), (s2, c2) in itertools.combinations(atoms, 2):
        enuc += ZNUC[s1] * ZNUC[s2] / np.linalg.norm(c1 - c2)
    E, eps, C = rhf(S, H, eri, nocc, enuc)
    mo_chem = np.einsum('pi,qj,pqrs,rk,sl->ijkl', C, C, eri, C, C, optimize=True)
    mo_phys = mo_chem.transpose(0, 2, 1, 3)
    return E, eps, mo_phys, eri, C


def pack_unique(eri_phys):
    """Unique (pq|rs) with p>=q, r>=s, pq>=rs (chemists' 8-fold symmetry)."""
    chem = eri_phys.transpose(0, 2, 1, 3)
    n = chem.shape[0]
    pq = [(p, q) for p in range(n) for q in range(p + 1)]
    vals = []
    for x, (p, q) in enumerate(pq):
        for (r, s) in pq[:x + 1]:
            vals.append(chem[p, q, r, s])
    return np.array(vals)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('SCESS_REFERENCE', '')
    basis = os.path.join(root, 'Assets', 'Basis')
    out = os.path.dirname(os.path.abspath(__file__))
    jobs = [('h2_sto3g', 'h2', os.path.join(basis, 'Pople', 'STO-3G.json'), 1),
            ('h2o_sto3g', 'h2o', os.path.join(basis, 'Pople', 'STO-3G.json'), 5),
            ('h2o_ccpvdz', 'h2o', os.path.join(basis, 'Dunning', 'cc-pVDZ.json'), 5)]
    for tag, mol, path, nocc in jobs:
        E, eps, eri, eri_ao, C = compute(mol, path, nocc)
        # AO integrals (chemists', normalised basis) and RHF coefficients C(mu, p):
        # inputs of the AO->MO transform, whose result is eri_unique
        np.savez_compressed(os.path.join(out, tag + '.npz'), E_RHF=E, eps=eps, nocc=nocc,
                            nmo=len(eps), eri_unique=pack_unique(eri),
                            ao_unique=pack_unique(eri_ao.transpose(0, 2, 1, 3)), C=C)
        print(f'{tag}: nmo={len(eps)} E(RHF) = {E:.10f}')


if __name__ == '__main__':
    main()
