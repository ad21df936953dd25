// Spin-orbital CCSD, CCSD-DIIS and (T) on the GPU: the cross-check solvers of
// SCESS (CCSD.cpp, CCSD-DIIS.cpp, CCSD_T.cpp), FP64 over engine einsums.
#pragma once
#include "engine.h"

namespace scess {

// <pq||rs> over 2n spin orbitals (spin orbital p = 2 x spatial + spin) from
// spatial chemists' integrals (PQ|RS) (n^4, column major):
// AntisymmetriseIntegrateOutSpinClosedShell, IntegralTransforms.cpp:135-162.
void so_antisymmetrise(Ctx &ctx, const double *d_chem, int64_t n, double *d_g);

struct SoResult {
  double E_CCSD = 0.0;  // 0 unless converged, as the reference's empty CCSD_Wfn
  double E_T = 0.0;
  double last_E = 0.0, last_dE = 0.0;
  int iterations = 0;
  bool converged = false;
};

// CCSD (CCSD.cpp:21-106), or CCSD_DIIS (CCSD-DIIS.cpp:17-198) when diis, from
// device <pq||rs> (N^4, N = 2 nmo) and spatial orbital energies (nmo); o = 2
// nocc spin-occupied orbitals.  d_t1 (o x v) and d_t2 (o x o x v x v, v = N -
// o) receive the final amplitudes.  With triples and a converged solve, E_T is
// CalculateTriplesCorrection of the result (CCSD_T, CCSD_T.cpp:18-66).
SoResult so_ccsd(Ctx &ctx, const double *d_g, const double *d_eps, int64_t nmo, int64_t nocc,
                 bool diis, bool triples, const Control &ctl, double *d_t1, double *d_t2);

// CalculateTriplesCorrection, CCSD_T.cpp:89-229 (spin-orbital t1, t2).
double so_triples(Ctx &ctx, const double *d_g, const double *d_eps, int64_t nmo, int64_t nocc,
                  const double *d_t1, const double *d_t2, const Control &ctl);

}  // namespace scess
