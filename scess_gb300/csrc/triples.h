// Closed-shell (T) correction on the GPU.
#pragma once
#include "engine.h"

namespace scess {

struct TriplesStats {
  int nb = 0;                 // virtual block size
  int64_t block_triples = 0;  // block triples processed
};

// E_(T) of RCCSD_TriplesCorrection (RCCSD_T.cpp:17-168) from device-resident
// eri (nmo^4, <pq|rs>), eps (nmo), t1 (o x v) and t2 (o x o x v x v).  With d_B
// (DF factors, naux x nmo x nmo) d_eri may be null: the integral slices (T)
// reads are formed from B directly and the nmo^4 eri is never built.
double rccsd_triples(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc,
                     const double *d_eps, const double *d_t1, const double *d_t2, bool mixed,
                     const Control &ctl, TriplesStats *stats = nullptr,
                     const double *d_B = nullptr, int64_t naux = 0);

// Gradient of E_(T) (no counterpart in the reference): adds
// gE * dE_T/dt1 (o x v) and gE * dE_T/dt2 (o x o x v x v) into d_gt1, d_gt2
// and, when d_geri is not null, gE * dE_T/deri (nmo^4, eri layout) into d_geri.
// Recomputes W per block triple, forms dE/dW and dE/dV in one FP64 kernel and
// runs the transposed GEMMs of the block: FP64 table GEMMs, or with `mixed`
// the same GEMMs on the tensor cores (split operands, FP32 accumulation).
// Returns E_(T).
double rccsd_triples_vjp(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc,
                         const double *d_eps, const double *d_t1, const double *d_t2, double gE,
                         const Control &ctl, double *d_gt1, double *d_gt2, double *d_geri,
                         bool mixed = false);

}  // namespace scess
