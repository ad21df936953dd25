// Closed-shell (T) correction on the GPU.
#pragma once
#include "engine.h"

namespace scess {

struct TriplesStats {
  int nb = 0;                 // virtual block size
  int64_t block_triples = 0;  // block triples processed
};

// E_(T) of RCCSD_TriplesCorrection (RCCSD_T.cpp:17-168) from device-resident
// eri (nmo^4, <pq|rs>), eps (nmo), t1 (o x v) and t2 (o x o x v x v).
double rccsd_triples(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc,
                     const double *d_eps, const double *d_t1, const double *d_t2, bool mixed,
                     const Control &ctl, TriplesStats *stats = nullptr);

}  // namespace scess
