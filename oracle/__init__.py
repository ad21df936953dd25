"""FP64 CPU oracle for the closed-shell CCSD / CCSD(T) path.

This package is TEST INFRASTRUCTURE. It restates, in NumPy float64, the
algorithm of SCESS's ``src/Quantum/CC/RCCSD.cpp`` (``SolveRCCSD_DIIS``) and
``src/Quantum/CC/RCCSD_T.cpp`` (``RCCSD_TriplesCorrection``) so that the CUDA
engine in ``scess_gb300`` can be checked against it.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
it; the product path never imports it.

Parity pinning: the restatement reproduces the reference's own known-answer
energies (``src/SCESS/Tests.cpp:34-75``) on H2/STO-3G, H2O/STO-3G and
H2O/cc-pVDZ integrals generated by ``tests/golden/make_molecules.py``.
"""
from .rccsd import (  # noqa: F401
    RCCSDIntegrals, make_integral_blocks, make_tau, plus_transpose,
    correlation_energy, coupling_energy, update_amplitudes, AmplitudeDIIS,
    solve_rccsd_diis, RCCSDWfn, full_piv_lu_solve, ccsd_flops,
)
from .rccsd_t import rccsd_triples_correction, triples_flops  # noqa: F401
from .f12 import f12b_coupling, contract_fixed_amplitudes  # noqa: F401
from .mp2 import mp2_energy, mp2_energy_ao  # noqa: F401
from .ccsd_so import (  # noqa: F401
    antisymmetrise_spin, ccsd as ccsd_spin_orbital, ccsd_t as ccsd_t_spin_orbital,
    triples_correction as spin_triples_correction,
)
