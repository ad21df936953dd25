// Closed-shell CCSD on the GPU: integral blocks, residual, Jacobi update, DIIS.
#pragma once
#include <deque>
#include <memory>
#include <vector>

#include "engine.h"

namespace scess {

// Particle ladder sum_cd <ab|cd> tau(i,j,c,d) in its symmetric /
// antisymmetric form: with V+-(ab,cd) = V(a,b,c,d) +- V(a,b,d,c) over pairs
// c <= d (c < d for -) and tau+- = (tau(i,j,c,d) +- tau(i,j,d,c)) / 2, the
// ladder is S(ij,ab) + -S-(ij,ab), S+- = tau+- V+-^T over pairs i <= j, a <= b
// (i < j, a < b for -): a quarter of the FLOPs of the plain contraction
// (it uses V(a,b,c,d) = V(b,a,d,c) and tau(i,j,c,d) = tau(j,i,d,c)).
struct LadderPM {
  int64_t nuo = 0, nso = 0, nuv = 0, nsv = 0;
  DevMem pairs;            // pu_o | ps_o | pu_v | ps_v as int2
  DTensor Vp, Vm;          // nuv x nuv, nsv x nsv (built once from the vvvv view)
  DTensor Tp, Tm, Sp, Sm;  // per call
  const int2 *pu_o = nullptr, *ps_o = nullptr, *pu_v = nullptr, *ps_v = nullptr;
};

// Integral blocks of RCCSD.cpp:32-44 as strided views into the device eri
// (no copies), plus the two materialised linear combinations.
struct RccsdBlocks {
  int64_t o = 0, v = 0, N = 0;
  TV ovov, oovv, ovvo, ovvv, ovoo, oooo, vvvv, oovv_phys;
  DTensor L_oovv, L_ovov;
  std::vector<DTensor> regions;  // DF build: the eri regions the views point into
  mutable std::unique_ptr<LadderPM> ladder;  // built on first use (ladder_pm)
  // The reassociated list's combined integrals, built on first use:
  // L_ovvv(k,d,a,c) = 2 (kd|ac) - (kc|ad), L_ovoo(l,c,k,i) = 2 (lc|ki) - (kc|li)
  mutable DTensor L_ovvv, L_ovoo;
  const TV &l_ovvv(Ctx &ctx) const;
  const TV &l_ovoo(Ctx &ctx) const;
  // views into the device eri (nmo^4)
  void build(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc);
  // from DF factors B (naux x nmo x nmo): only the seven regions of <pq|rs> the
  // views need are contracted (no nmo^4 tensor); be: FP64 or the tensor cores
  void build_df(Ctx &ctx, const double *d_B, int64_t naux, int64_t nmo, int64_t nocc,
                Backend be);

 private:
  void build_l(Ctx &ctx);
};

// Device work arrays of one residual evaluation.
struct RccsdWork {
  DTensor tau, Foo, Fvv, Fov, Fovt1, Loo, Lvv, X, tmp_abic, tmp_kibj, tmp_akij, Woooo, Wvvvv,
      Wvoov, Wvovo, tmp_lkci, tmp_lcki, Yd;
  void alloc(int64_t o, int64_t v, bool direct_vvvv);
};

// R1(i,a), R2(i,j,a,b): the numerators t1new, t2new of UpdateAmplitudes
// (RCCSD.cpp:101-233) before the division by the denominators (:235-236).
// amp = [t1 | t2] and R = [R1 | R2] (column major).  Backend::FP64 follows the
// reference's contraction list literally; Backend::MIXED evaluates the large
// contractions on tensor cores and folds the T1 dressing of Wvvvv into the
// ladder (vvvv tau plus two o^3v^3 contractions), so no v^4 tensor is formed.
// list: the reference's literal contraction list (AUTO for the FP64 backend:
// the drop-in path) or the reassociated one (AUTO for the tensor cores; also
// the FP64 base evaluations of the refined mixed solve, which then write no
// v^4 tensor).  Both compute the same function.
enum class ResidualList { AUTO = 0, LITERAL = 1, REASSOCIATED = 2 };
void rccsd_residual(Ctx &ctx, const RccsdBlocks &B, const double *amp, const double *t2driver,
                    Backend be, RccsdWork &w, double *R, ResidualList list = ResidualList::AUTO);

// R2 += sum_cd <ab|cd> tau(i,j,c,d) through the symmetric / antisymmetric
// form (LadderPM), on the backend be; the V+- operands are built from the
// vvvv view on first use and kept with the blocks.
void ladder_pm(Ctx &ctx, const RccsdBlocks &B, const TV &tau, double *R2, Backend be);

// Change of the residual numerators, dR = R(T0 + d) - R(T0), for the
// reassociated list: w0 holds that list's intermediates at T0 (from
// rccsd_residual with the reassociated list, FP64), amp1 = T0 + d and
// damp = d.  Every product is expanded so that it has a factor of the size of
// d (A1 B1 - A0 B0 = dA B1 + A0 dB), so the rounding error of the tensor-core
// contractions scales with |d|, not with |T|: R0 + dR is then as accurate as
// an FP64 evaluation while |d| stays small.  w receives the changes of the
// intermediates; tau1 (o^2 v^2) is scratch.
void rccsd_residual_delta(Ctx &ctx, const RccsdBlocks &B, const double *amp0, const double *amp1,
                          const double *damp, const RccsdWork &w0, Backend be, RccsdWork &w,
                          double *tau1, double *dR);

struct SolveInput {
  const double *eps_host = nullptr;     // nmo
  const double *f12_residual = nullptr; // host o^2v^2 or null
  const double *f12_energy = nullptr;   // host o^2v^2 or null
};

// Device-resident CCSD problem: integrals (eri + block views), orbital
// energies, amplitudes and the DIIS subspace stay in HBM between calls.
// iterate() runs the loop body of SolveRCCSD_DIIS (RCCSD.cpp:345-374).
class RccsdState {
 public:
  RccsdState(Ctx &ctx, DTensor &&eri, int64_t nmo, int64_t nocc, const SolveInput &in,
             const scess_rccsd_options &opts);
  // DF state: B (naux x nmo x nmo) on the device; no nmo^4 eri is formed
  RccsdState(Ctx &ctx, DTensor &&B, int64_t naux, int64_t nmo, int64_t nocc,
             const SolveInput &in, const scess_rccsd_options &opts);
  ~RccsdState();
  void mp2_guess();
  void set_amplitudes(const double *t1, const double *t2);
  void get_amplitudes(double *t1, double *t2);
  // Up to max_steps iterations (fewer once converged); returns converged.
  bool iterate(int max_steps, const Control &ctl);
  double coupling_energy();
  double energy_of_amplitudes();
  const scess_rccsd_result &result() const { return res_; }
  const scess_rccsd_options &options() const { return opts_; }
  bool has_f12() const { return have_f12_; }
  float last_device_ms() const { return last_device_ms_; }
  const RccsdBlocks &blocks() const { return B_; }
  const double *d_eri() const { return eri_.p(); }  // null for a DF state
  const double *d_B() const { return dfB_.p(); }     // null unless a DF state
  int64_t naux() const { return naux_; }
  const double *d_eps() const { return eps_.p(); }
  const double *d_t1() const { return amp_.p(); }
  const double *d_t2() const { return amp_.p() + n1_; }
  int64_t nocc() const { return B_.o; }
  int64_t nmo() const { return B_.N; }

 private:
  void reset_history();
  void init(const SolveInput &in, const scess_rccsd_options &opts);
  Ctx &ctx_;
  DTensor eri_;
  DTensor dfB_;
  int64_t naux_ = 0;
  RccsdBlocks B_;
  scess_rccsd_options opts_;
  int64_t n1_ = 0, n2_ = 0, n_ = 0;
  bool mixed_ = false, have_f12_ = false, have_wvvvv_ = false;
  DTensor eps_, amp_, prev_, R_, drv_, Lf12_;
  int maxv_ = 8;
  DevMem diis_amp_, diis_err_, vecptr_, coefd_;
  RccsdWork w_;
  std::deque<int> order_;  // DIIS slots, oldest first
  std::vector<std::vector<double>> gram_;
  double E_last_ = 0.0;
  // Phases of a solve.  FP64: every iteration in FP64 (the drop-in path).  A
  // MIXED solve: MIXED (tensor-core residuals) until its switch thresholds;
  // BASE, one FP64 iteration whose residual R0 and intermediates at its input
  // amplitudes T0 are kept; REFINED, iterations whose residual is
  // R0 + dR(T0, T - T0) (rccsd_residual_delta, tensor cores) until the
  // reference's criteria hold; CONFIRM, an FP64 iteration that must meet
  // them too, else it becomes the new base and REFINED resumes.
  enum class Phase { FP64, MIXED, BASE, REFINED, CONFIRM };
  Phase phase_ = Phase::FP64;
  RccsdWork w0_;                       // intermediates at the base amplitudes
  DTensor amp0_, R0_, damp_, tau1_;    // base amplitudes and residual; change; scratch
  int it_ = 0, phase_start_ = 0, fp64_iters_ = 0;
  bool converged_ = false;
  scess_rccsd_result res_{};
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  float last_device_ms_ = 0.0f;
};

// SolveRCCSD_DIIS (RCCSD.cpp:295-394) on a prepared state.
void rccsd_solve(Ctx &ctx, RccsdState &st, const Control &ctl, double *t1_out, double *t2_out,
                 scess_rccsd_result *res);

// Host-side DIIS solve with the reference's semantics (RCCSD.cpp:246-274):
// bordered Gram matrix scaled by max|B|, full-pivoting LU.
std::vector<double> diis_coefficients(const std::vector<std::vector<double>> &gram);
// Full-pivoting LU solve (Eigen FullPivLU::solve behaviour), row-major n x n.
std::vector<double> full_piv_lu_solve(std::vector<double> A, std::vector<double> b, int n);

}  // namespace scess
