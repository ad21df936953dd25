"""GB300-native closed-shell CCSD / CCSD(T) engine (sm_103a CUDA behind a C ABI).

The product is ``libscess_cc.so`` (built by :mod:`scess_gb300.build`); this
package exposes its C ABI through :mod:`scess_gb300.cc`, whose
``SolveRCCSD_DIIS`` / ``RCCSD_TriplesCorrection`` mirror SCESS's
``src/Quantum/CC/CC.h`` interface.
"""
from .cc import (  # noqa: F401
    Context, RCCSD_Wfn, RCCSD_F12Coupling, ScessError, SolveRCCSD_DIIS,
    RCCSD_TriplesCorrection, load_library, EXPORTS, LIB_PATH,
    CCSD_Wfn, CCSD, CCSD_DIIS, CCSD_T, CalculateTriplesCorrection,
)
