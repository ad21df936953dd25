"""Test infrastructure: NumPy float64 restatement of SCESS's closed-shell MP2,
``src/Quantum/HF/RHF.cpp:267-345`` (MP2_RHF_ClosedShellAO, MP2_RHF_ClosedShell).
Only the tests may use it.  Pinned on the reference's MP2 energies
(``Tests.cpp:37,42,51``, checked at ``:546-548, :567-569, :601-603``)."""
import numpy as np


def mp2_energy(mo_chem, eps, nocc):
    """MP2_RHF_ClosedShell, RHF.cpp:324-340: mo_chem(p,q,r,s) = (pq|rs)."""
    o = int(nocc)
    g = mo_chem[:o, o:, :o, o:]                      # (ia|jb)
    e = np.asarray(eps)
    d = e[o:][None, :, None, None] + e[o:][None, None, None, :] - e[:o][:, None, None, None] \
        - e[:o][None, None, :, None]
    return float(-np.sum(g * (2.0 * g - g.transpose(0, 3, 2, 1)) / d))


def mp2_energy_ao(ao_chem, C, eps, nocc):
    """MP2_RHF_ClosedShellAO, RHF.cpp:281-296: (a i|b j) from the AO integrals."""
    o = int(nocc)
    Co, Cv = C[:, :o], C[:, o:]
    aibj = np.einsum('mnkl,ma,ni,kb,lj->aibj', ao_chem, Cv, Co, Cv, Co, optimize=True)
    e = np.asarray(eps)
    d = e[o:][:, None, None, None] + e[o:][None, None, :, None] - e[:o][None, :, None, None] \
        - e[:o][None, None, None, :]
    ibja = aibj.transpose(2, 1, 0, 3)                 # aibj(b, i, a, j)
    return float(-np.sum(aibj * (2.0 * aibj - ibja) / d))
