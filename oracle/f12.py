"""Test infrastructure: NumPy float64 restatement of the CCSD-F12b coupling of
SCESS's ``src/Quantum/F12/CCSD_F12b.cpp`` (the part that feeds
``SolveRCCSD_DIIS``).  Only the tests may use it.

Parity is unpinned for this piece: the reference's CCSD-F12b pins
(``Tests.cpp:72-74,675-680``) need its MP2-F12/3C intermediates and CABS
integrals, which are outside this engine; the restatement follows the
reference's code line by line instead.
"""
import numpy as np


def contract_fixed_amplitudes(X):
    """ContractFixedAmplitudes, CCSD_F12b.cpp:31-35: sum_kl c_ij^kl X_kl^ab with
    the SP geminal amplitudes, = 3/8 X_ij^ab + 1/8 X_ji^ab, indexed (i, j, a, b)."""
    return 0.375 * X + 0.125 * X.transpose(1, 0, 2, 3)


def f12b_coupling(eri, f12, f12_repulsion, C, nocc):
    """CCSD_F12b.cpp:83-91.  eri, f12, f12_repulsion: nmo^4 OBS tensors in
    physicists' notation; C: the MP2-F12/3C intermediate (o, o, v, v).
    Returns (residual, energy) of RCCSD_F12Coupling, both (o, o, v, v)."""
    o = int(nocc)
    # V_klab = <kl| r12^-1 f12 |ab> - sum_rs <ab|rs><kl|f12|rs>              :85-87
    V = f12_repulsion[:o, :o, o:, o:].copy()
    V -= np.einsum('abrs,klrs->klab', eri[o:, o:, :, :], f12[:o, :o, :, :], optimize=True)
    residual = contract_fixed_amplitudes(C + V)                                # :90
    energy = contract_fixed_amplitudes(C)                                      # :91
    return residual, energy
