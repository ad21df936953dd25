// Closed-shell CCSD on the GPU: integral blocks, residual, Jacobi update, DIIS.
#pragma once
#include <deque>
#include <vector>

#include "engine.h"

namespace scess {

// Integral blocks of RCCSD.cpp:32-44 as strided views into the device eri
// (no copies), plus the two materialised linear combinations.
struct RccsdBlocks {
  int64_t o = 0, v = 0, N = 0;
  TV ovov, oovv, ovvo, ovvv, ovoo, oooo, vvvv, oovv_phys;
  DTensor L_oovv, L_ovov;
  void build(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc);
};

// Device work arrays of one residual evaluation.
struct RccsdWork {
  DTensor tau, Foo, Fvv, Fov, Fovt1, Loo, Lvv, X, tmp_abic, tmp_akij, Woooo, Wvvvv, Wvoov,
      Wvovo, tmp_lkci, tmp_lcki, Yd;
  void alloc(int64_t o, int64_t v, bool direct_vvvv);
};

// R1(i,a), R2(i,j,a,b): the numerators t1new, t2new of UpdateAmplitudes
// (RCCSD.cpp:101-233) before the division by the denominators (:235-236).
// amp = [t1 | t2] and R = [R1 | R2] (column major).  Backend::FP64 follows the
// reference's contraction list literally; Backend::MIXED evaluates the large
// contractions on tensor cores and folds the T1 dressing of Wvvvv into the
// ladder (vvvv tau plus two o^3v^3 contractions), so no v^4 tensor is formed.
void rccsd_residual(Ctx &ctx, const RccsdBlocks &B, const double *amp, const double *t2driver,
                    Backend be, RccsdWork &w, double *R);

// Full solver (SolveRCCSD_DIIS, RCCSD.cpp:295-394) on device-resident blocks.
struct SolveInput {
  const double *eps_host = nullptr;     // nmo
  const double *f12_residual = nullptr; // host o^2v^2 or null
  const double *f12_energy = nullptr;   // host o^2v^2 or null
};
void rccsd_solve(Ctx &ctx, const RccsdBlocks &B, const SolveInput &in,
                 const scess_rccsd_options &opts, const Control &ctl, double *t1_out,
                 double *t2_out, scess_rccsd_result *res);

// Host-side DIIS solve with the reference's semantics (RCCSD.cpp:246-274):
// bordered Gram matrix scaled by max|B|, full-pivoting LU.
std::vector<double> diis_coefficients(const std::vector<std::vector<double>> &gram);
// Full-pivoting LU solve (Eigen FullPivLU::solve behaviour), row-major n x n.
std::vector<double> full_piv_lu_solve(std::vector<double> A, std::vector<double> b, int n);

}  // namespace scess
