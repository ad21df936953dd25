/*
 * scess_cc.h - C ABI of the GB300-native closed-shell CCSD / CCSD(T) engine.
 *
 * Drop-in for SCESS's closed-shell coupled-cluster calls:
 *   RCCSD_Wfn SolveRCCSD_DIIS(const TEITensor &eri, const VectorXd &orbitalEnergies,
 *                             Index nOcc, const RCCSD_F12Coupling *f12,
 *                             const DH::Thread *thread, std::stringstream *console)
 *       declared src/Quantum/CC/CC.h:136-141, defined src/Quantum/CC/RCCSD.cpp:295-394
 *   double RCCSD_TriplesCorrection(const TEITensor &eri, const VectorXd &orbitalEnergies,
 *                                  Index nOcc, const T1Tensor &t1, const T2Tensor &t2,
 *                                  const DH::Thread *thread)
 *       declared src/Quantum/CC/CC.h:154-158, defined src/Quantum/CC/RCCSD_T.cpp:17-168
 *
 * Conventions (identical to the reference's Eigen tensors):
 *   - every array is a caller-owned HOST buffer of doubles in COLUMN-MAJOR order
 *     (first index fastest), exactly the memory of an Eigen::Tensor<double,k>;
 *   - eri(p,q,r,s) = <pq|rs> = (pr|qs) over nmo spatial MOs, occupied first;
 *   - t1(i,a) is o x v, t2(i,j,a,b) is o x o x v x v with t2(i,j,a,b) = t2(j,i,b,a);
 *   - DF factors B(Q,p,q) are naux x nmo x nmo, symmetric in (p,q), with
 *     (pq|rs) = sum_Q B(Q,p,q) B(Q,r,s).
 *
 * Every call is synchronous and returns an SCESS_* status.  A context owns one
 * GPU's device memory and stream; use one context per calling thread.
 * Non-convergence is not an error (result.converged = 0, as the reference).
 */
#ifndef SCESS_CC_H
#define SCESS_CC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference signals cancellation by returning an empty
 * wavefunction / 0.0 (RCCSD.cpp:346-347, RCCSD_T.cpp:161-162); here it is
 * SCESS_ERR_CANCELLED. */
#define SCESS_OK 0
#define SCESS_ERR_INVALID 1     /* bad shape, null pointer, NaN/Inf input      */
#define SCESS_ERR_OOM 2         /* device (or pinned host) allocation failed   */
#define SCESS_ERR_CUDA 3        /* CUDA runtime / launch failure               */
#define SCESS_ERR_CANCELLED 4   /* cancel callback returned non-zero           */
#define SCESS_ERR_TIMEOUT 5     /* options.time_limit_s exceeded               */
#define SCESS_ERR_UNSUPPORTED 6 /* no sm_103a device / feature not available   */
#define SCESS_ERR_TOO_LARGE 7   /* scess_einsum_static: beyond its fixed scratch */

/* Arithmetic of the contractions. FP64 is the drop-in path (matches the
 * reference to <= 1e-9 Eh); MIXED runs the contractions on FP16 tensor cores
 * (tcgen05, split hi+lo operands, FP32 accumulation) with FP64 denominators,
 * DIIS and energies, followed by a refinement that ends in FP64 iterations
 * (see refine_sweeps). */
#define SCESS_PRECISION_FP64 0
#define SCESS_PRECISION_MIXED 1

typedef struct scess_ctx scess_ctx;

/* Polled between phases; non-zero stops the call with SCESS_ERR_CANCELLED.
 * Replaces DH::Thread::ShouldStop() (RCCSD.cpp:346, RCCSD_T.cpp:123). */
typedef int (*scess_cancel_fn)(void *user);
/* Receives the per-iteration console lines of RCCSD.cpp:312-392
 * ("CCSD(n): E(corr) = ... dE = ... rms(dt) = ..."). */
typedef void (*scess_log_fn)(int level, const char *message, void *user);

/* Options of SolveRCCSD_DIIS. Defaults (scess_rccsd_default_options) are the
 * reference's compile-time constants, RCCSD.cpp:302-307. */
typedef struct {
  double energy_convergence;    /* 1e-10 */
  double amplitude_convergence; /* 1e-8  */
  int32_t max_iterations;       /* 100   */
  int32_t diis_start;           /* 2     */
  int32_t max_diis_vectors;     /* 8     */
  int32_t precision;            /* SCESS_PRECISION_FP64 */
  /* MIXED only: the least number of FP64 iterations of the refinement (at
   * least 1).  The refinement starts with one FP64 iteration (the base: its
   * residual R0 and intermediates at its amplitudes T0 are kept), continues
   * with refined iterations whose residual R0 + dR(T0, T - T0) runs on the
   * tensor cores with every product carrying a factor of the size of T - T0
   * (so its rounding error shrinks with T - T0), and ends with an FP64
   * iteration that must meet the convergence criteria (else it becomes the
   * new base).  The returned energy comes from that FP64 iteration. */
  int32_t refine_sweeps;        /* 2 */
  /* MIXED only: the mixed phase ends once dE < mixed_energy_switch and
   * rms(dt) < mixed_amplitude_switch; the refinement then starts from the
   * mixed amplitudes with a fresh DIIS subspace. */
  double mixed_energy_switch;     /* 1e-8 */
  double mixed_amplitude_switch;  /* 1e-6 */
  /* 0: MP2 initial guess (RCCSD.cpp:333-339). 1: resume from the amplitudes
   * passed in t1_out / t2_out (e.g. a checkpoint). */
  int32_t resume;               /* 0 */
  /* Optional per-iteration amplitude checkpoint ring on the host: iteration n
   * writes slot n % capacity (o*v and o^2*v^2 doubles per slot). */
  double *checkpoint_t1;
  double *checkpoint_t2;
  int32_t checkpoint_capacity;
  /* Optional: 3 doubles per iteration (E, dE, rms) for max_iterations rows. */
  double *history;
  /* Wall-clock limit of the call in seconds (0 = none) -> SCESS_ERR_TIMEOUT. */
  double time_limit_s;
} scess_rccsd_options;

/* RCCSD_Wfn (CC.h:105-115) minus the tensors, which go to t1_out / t2_out. */
typedef struct {
  double E_CCSD;          /* correlation energy incl. the F12 coupling energy */
  double E_F12_Coupling;  /* CouplingEnergy(f12, t2) (RCCSD.cpp:91-98)         */
  double E_T;             /* set by scess_rccsd_triples only                  */
  int32_t converged;
  int32_t iterations;     /* total iterations run (mixed + FP64)              */
  int32_t mixed_iterations; /* iterations whose residual ran on the tensor cores */
  double last_dE;
  double last_rms;
  int32_t fp64_iterations;  /* iterations with an FP64 residual               */
} scess_rccsd_result;

const char *scess_status_string(int status);
/* Number of CUDA kernels this library has launched in the process so far. */
int64_t scess_launch_count(void);

/* Context on CUDA device `device` (must be sm_103a). */
int scess_ctx_create(int device, scess_ctx **out);
void scess_ctx_destroy(scess_ctx *ctx);
/* Message of the last failing call on this context ("" if none). */
const char *scess_ctx_last_error(const scess_ctx *ctx);
int scess_ctx_set_callbacks(scess_ctx *ctx, scess_cancel_fn cancel, scess_log_fn log, void *user);

/* Device-memory cap of a context (no counterpart in the reference, which runs
 * on host memory).  For a GPU shared with other work: the device memory this
 * context's calls hold (their live buffers and the context's cache of released
 * blocks) stays within `bytes`; an allocation beyond it first empties the
 * cache, then fails with SCESS_ERR_OOM as a full device would, and the context
 * stays usable.  0 removes the cap.  scess_ctx_memory_held reports the bytes
 * currently held (-1 for a bad context). */
int scess_ctx_set_memory_limit(scess_ctx *ctx, int64_t bytes);
int64_t scess_ctx_memory_held(const scess_ctx *ctx);

/* Diagnostics of the tensor-core kernels' failure path (no counterpart in the
 * reference).  Every pipeline wait inside those kernels is bounded; this arms
 * the NEXT tensor-core launch of the context with a bound of `wait_cycles` GPU
 * clock cycles (2^16 .. 2^40; production launches use ~2^32) and makes its
 * copy thread leave the first operand stage unfilled, so that the MMA
 * thread's wait on it runs out.  The kernel then records the expiry, lets the
 * copies it did issue land, frees its tensor memory and returns; the call that
 * made the launch fails with SCESS_ERR_CUDA ("tensor-core pipeline wait
 * expired"), and later calls on the context run normally.  Nothing faults,
 * traps or hangs. */
int scess_ctx_arm_wait_expiry(scess_ctx *ctx, int64_t wait_cycles);

void scess_rccsd_default_options(scess_rccsd_options *opts);

/* SolveRCCSD_DIIS (CC.h:136-141, RCCSD.cpp:295-394).
 *   eri          nmo^4, <pq|rs>
 *   eps          nmo orbital energies
 *   f12_residual RCCSD_F12Coupling::residual (o^2 v^2) or NULL  (CC.h:121-124)
 *   f12_energy   RCCSD_F12Coupling::energy   (o^2 v^2) or NULL
 *   t1_out       o*v   converged t1 (also the resume input when opts->resume)
 *   t2_out       o^2 v^2 converged t2
 * On non-convergence result->converged = 0, energies are 0 and t1/t2 are left
 * unchanged, as RCCSD.cpp:376-380. opts may be NULL (defaults). */
int scess_rccsd_solve(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                      int64_t nocc, const double *f12_residual, const double *f12_energy,
                      const scess_rccsd_options *opts, double *t1_out, double *t2_out,
                      scess_rccsd_result *result);

/* Same as scess_rccsd_solve, from DF factors B (naux x nmo x nmo): only the
 * regions of <pq|rs> the integral blocks read are contracted from B on the GPU
 * (on the tensor cores for SCESS_PRECISION_MIXED); no nmo^4 eri is formed. */
int scess_rccsd_solve_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                         int64_t nmo, int64_t nocc, const double *f12_residual,
                         const double *f12_energy, const scess_rccsd_options *opts,
                         double *t1_out, double *t2_out, scess_rccsd_result *result);

/* RCCSD_TriplesCorrection (CC.h:154-158, RCCSD_T.cpp:17-168): E_(T) into *e_t.
 * precision: SCESS_PRECISION_FP64 (drop-in) or SCESS_PRECISION_MIXED. */
int scess_rccsd_triples(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                        int64_t nocc, const double *t1, const double *t2, int32_t precision,
                        double *e_t);

/* (T) from DF factors B (naux x nmo x nmo, (pq|rs) = sum_Q B(Q,p,q) B(Q,r,s)):
 * the only integrals (T) reads, (ia|bf), (ia|mj) and (ia|jb), are contracted
 * from B on the device (FP64, or on the tensor cores for MIXED); the nmo^4
 * eri is never formed. */
int scess_rccsd_triples_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                           int64_t nmo, int64_t nocc, const double *t1, const double *t2,
                           int32_t precision, double *e_t);

/* ---- Device-resident session (no counterpart call in the reference: SCESS
 * keeps these objects inside SolveRCCSD_DIIS, RCCSD.cpp:318-344).  The
 * integrals, orbital energies, amplitudes (MP2 guess, RCCSD.cpp:333-339) and
 * the DIIS subspace stay in GPU memory between calls, so a caller can step the
 * iteration, run (T) on the current amplitudes and read them back without
 * re-sending the nmo^4 integrals. */
typedef struct scess_rccsd_state scess_rccsd_state;

int scess_rccsd_state_create(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                             int64_t nocc, const double *f12_residual, const double *f12_energy,
                             const scess_rccsd_options *opts, scess_rccsd_state **out);
/* DF state: keeps B and the integral regions contracted from it (no nmo^4
 * eri); scess_rccsd_state_triples on it forms the (T) slices from B. */
int scess_rccsd_state_create_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                                int64_t nmo, int64_t nocc, const double *f12_residual,
                                const double *f12_energy, const scess_rccsd_options *opts,
                                scess_rccsd_state **out);
void scess_rccsd_state_destroy(scess_rccsd_state *state);
/* Runs up to n_iterations of the SolveRCCSD_DIIS loop (RCCSD.cpp:345-374),
 * fewer once converged; *device_ms (optional) is the GPU time of the call
 * measured with CUDA events on the context's stream. */
int scess_rccsd_state_iterate(scess_rccsd_state *state, int32_t n_iterations,
                              scess_rccsd_result *result, double *device_ms);
/* E_(T) (RCCSD_T.cpp:17-168) from the state's current amplitudes. */
int scess_rccsd_state_triples(scess_rccsd_state *state, int32_t precision, double *e_t,
                              double *device_ms);
int scess_rccsd_state_amplitudes(scess_rccsd_state *state, double *t1_out, double *t2_out);
int scess_rccsd_state_set_amplitudes(scess_rccsd_state *state, const double *t1,
                                     const double *t2);

/* Kernel timing on the context's stream (CUDA events around each launch of
 * the engine's GEMM, pack and (T) kernels).  enable != 0 clears and starts,
 * 0 stops.  The report is a JSON object {kernel: {"launches", "ms", "flops",
 * "bytes"}} written into buf (truncated to buflen). */
int scess_ctx_profile(scess_ctx *ctx, int32_t enable);
int scess_ctx_profile_report(scess_ctx *ctx, char *buf, int64_t buflen);

/* One UpdateAmplitudes residual (RCCSD.cpp:101-233) without the final division
 * by the denominators (:235-236): r1_out = t1new (o*v), r2_out = t2new
 * (o^2 v^2), so that t1 <- r1/eia and t2 <- r2/eijab is the reference's
 * update.  t2_driver is RCCSD_F12Coupling::residual or NULL. */
int scess_rccsd_residual(scess_ctx *ctx, const double *eri, int64_t nmo, int64_t nocc,
                         const double *t1, const double *t2, const double *t2_driver,
                         int32_t precision, double *r1_out, double *r2_out);
/* Same from DF factors B (naux x nmo x nmo): the forward half of the pair
 * whose reverse is scess_rccsd_residual_vjp_df; the eri
 * <pq|rs> = sum_Q B(Q,p,r) B(Q,q,s) is formed on the GPU in FP64. */
int scess_rccsd_residual_df(scess_ctx *ctx, const double *B, int64_t naux, int64_t nmo,
                            int64_t nocc, const double *t1, const double *t2,
                            const double *t2_driver, int32_t precision, double *r1_out,
                            double *r2_out);

/* Vector-Jacobian product of the residual numerators R(t1, t2; eri) of
 * scess_rccsd_residual (UpdateAmplitudes, RCCSD.cpp:101-233; the reference has
 * no derivative code).  Given cotangents g_r1 (o*v) and g_r2 (o^2 v^2):
 *   g_t1 = (dR/dt1)^T g_r, g_t2 = (dR/dt2)^T g_r, g_eri = (dR/deri)^T g_r
 * (g_eri nmo^4, may be NULL).  Hand-written reverse sweep over the forward's
 * recorded contractions, on the GPU.  precision FP64 or MIXED (the
 * contractions of forward and adjoint on tensor cores, FP32 accumulation). */
int scess_rccsd_residual_vjp(scess_ctx *ctx, const double *eri, int64_t nmo, int64_t nocc,
                             const double *t1, const double *t2, const double *g_r1,
                             const double *g_r2, int32_t precision, double *g_t1, double *g_t2,
                             double *g_eri);
/* Same from DF factors; g_B (naux x nmo x nmo, may be NULL) = (dR/dB)^T g_r. */
int scess_rccsd_residual_vjp_df(scess_ctx *ctx, const double *B, int64_t naux, int64_t nmo,
                                int64_t nocc, const double *t1, const double *t2,
                                const double *g_r1, const double *g_r2, int32_t precision,
                                double *g_t1, double *g_t2, double *g_B);

/* Vector-Jacobian product of E_(T) (RCCSD_TriplesCorrection, RCCSD_T.cpp:17-168;
 * the reference has no derivative code): for a cotangent g_e, writes
 * g_e dE_T/dt1 (o*v), g_e dE_T/dt2 (o^2 v^2) and, when g_eri is not NULL,
 * g_e dE_T/deri (nmo^4, eri layout; nonzero only on the (ov|vv), (oo|vo) and
 * (ov|ov) blocks E_T reads).  e_t (may be NULL) receives E_T.  The forward
 * W is recomputed block by block, so the memory use is that of the FP64 (T).
 * precision: SCESS_PRECISION_FP64 (FP64 table GEMMs), or MIXED (the forward
 * and transposed GEMMs on the tensor cores: split operands, FP32
 * accumulation; the element-wise gradient of the energy stays FP64). */
int scess_rccsd_triples_vjp(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                            int64_t nocc, const double *t1, const double *t2, int32_t precision,
                            double g_e, double *e_t, double *g_t1, double *g_t2, double *g_eri);
/* Same from DF factors; g_B (naux x nmo x nmo, may be NULL) = g_e dE_T/dB. */
int scess_rccsd_triples_vjp_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                               int64_t nmo, int64_t nocc, const double *t1, const double *t2,
                               int32_t precision, double g_e, double *e_t, double *g_t1,
                               double *g_t2, double *g_B);

/* CCSD Lambda (left-hand) equations at converged t1/t2 (no counterpart in the
 * reference).  Omega(t; f) is the closed-shell residual with the Fock terms that
 * UpdateAmplitudes drops for canonical orbitals (RCCSD.cpp:13-15, :109), the
 * energy is E = 2 sum f_ia t_ia + sum L_oovv tau, and lambda solves
 * dE/dt + (dOmega/dt)^T lambda = 0 on the closed-shell subspace
 * t2(ijab) = t2(jiba) (l1: o*v, l2: o^2 v^2, l2 symmetric likewise).  Each iteration is
 * one reverse sweep of the recorded residual on the GPU, with DIIS as in
 * AmplitudeDIIS; convergence: rms(dlambda) < opts->amplitude_convergence.
 * result->converged / iterations / last_rms are set. */
int scess_rccsd_lambda(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                       int64_t nocc, const double *t1, const double *t2,
                       const scess_rccsd_options *opts, double *l1_out, double *l2_out,
                       scess_rccsd_result *result);
/* Unrelaxed one-particle density (correlation part, spin-summed, MO basis,
 * nmo x nmo symmetric, column-major): gamma_pq = dL/df_pq of the Lagrangian
 * above, so that dE_CCSD = sum_pq gamma_pq df_pq for a symmetric change of the
 * Fock matrix at fixed orbitals. */
int scess_rccsd_rdm1(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                     int64_t nocc, const double *t1, const double *t2, const double *l1,
                     const double *l2, int32_t precision, double *dm1_out);

/* General binary contraction C = alpha * A.B + beta * C on the GPU, the
 * runtime counterpart of the tensor layer's compile-time Einsum
 * (src/Tensor/TensorEinsum.h:170-205): spec like "kcld,ilcd->ki", each
 * operand a dense column-major host tensor of rank <= 6 with extents *_ext.
 * Every label of C appears in exactly one of A, B; labels shared by A and B
 * and absent from C are summed.  precision selects the FP64 (DFMA) backend
 * or, for MIXED, the tcgen05 tensor-core backend for any shape. */
int scess_einsum(scess_ctx *ctx, const char *spec, double alpha, const double *A, int32_t a_nd,
                 const int64_t *a_ext, const double *B, int32_t b_nd, const int64_t *b_ext,
                 double beta, double *C, int32_t c_nd, const int64_t *c_ext, int32_t precision);

/* AO->MO transform of the two-electron integrals, TransformTEI
 * (src/Quantum/Integrals/IntegralTransforms.cpp:32-59): tei is the chemists'
 * AO tensor (mu nu|kap lam) (nao^4, column-major); A, B, C, D are AO x MO
 * coefficient matrices (nao x na, ..., column-major).  out(p,q,r,s) =
 * sum A(mu,p) B(nu,q) C(kap,r) D(lam,s) (mu nu|kap lam), transformed one index
 * at a time (lam, kap, nu, mu) as the reference does; with chem_to_phys the
 * result is reordered pqrs -> prqs (out is then na x nc x nb x nd), which with
 * A = B = C = D is the physicists' eri of scess_rccsd_solve (RCCSD.cpp:399).
 * precision: FP64 table GEMMs, or MIXED (tensor cores, split operands). */
int scess_transform_tei(scess_ctx *ctx, const double *tei, int64_t nao, const double *A,
                        int64_t na, const double *B, int64_t nb, const double *C, int64_t nc,
                        const double *D, int64_t nd, int32_t chem_to_phys, int32_t precision,
                        double *out);

/* CCSD-F12b coupling of the conventional doubles to the fixed-amplitude
 * geminals, CCSD_F12b.cpp:83-94 (the part of CCSD_F12b that feeds
 * SolveRCCSD_DIIS).  All tensors are over the nmo OBS MOs, occupied first,
 * physicists' notation, column-major: eri <pq|rs>, f12 <pq|f12|rs>,
 * f12_repulsion <pq|r12^-1 f12|rs> (nmo^4 each), and C the MP2-F12/3C
 * intermediate C_kl^ab (nocc^2 nvirt^2).  With
 *   V(k,l,a,b) = f12_repulsion(k,l,a,b) - sum_rs eri(a,b,r,s) f12(k,l,r,s)
 * and F(X)(i,j,a,b) = 3/8 X(i,j,a,b) + 1/8 X(j,i,a,b) (ContractFixedAmplitudes),
 * residual_out = F(C + V) and energy_out = F(C) (nocc^2 nvirt^2 each): the
 * f12_residual and f12_energy arguments of scess_rccsd_solve.  precision:
 * FP64 (table GEMM), or MIXED (the rs contraction on tensor cores). */
int scess_f12b_coupling(scess_ctx *ctx, const double *eri, const double *f12,
                        const double *f12_repulsion, const double *C, int64_t nmo, int64_t nocc,
                        int32_t precision, double *residual_out, double *energy_out);

/* Closed-shell MP2 correlation energy, MP2_RHF_ClosedShell (RHF.cpp:306-345):
 * E = -sum_ijab (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_a + e_b - e_i - e_j) from
 * the CHEMISTS'-notation MO tensor mo_eri(p,q,r,s) = (pq|rs) (nmo^4,
 * column-major, occupied first) and the orbital energies eps (nmo).  FP64. */
int scess_mp2_energy(scess_ctx *ctx, const double *mo_eri, const double *eps, int64_t nmo,
                     int64_t nocc, double *e_mp2);

/* MP2 from AO integrals, MP2_RHF_ClosedShellAO (RHF.cpp:267-304): ao_eri is
 * (mu nu|kap lam) (nao^4), C the MO coefficients (nao x nmo, occupied first),
 * eps (nmo); (a i|b j) is formed with scess_transform_tei's quarter transforms
 * (C_virt, C_occ, C_virt, C_occ) and summed as the reference does.
 * precision: FP64, or MIXED for the transform (the sum is FP64). */
int scess_mp2_energy_ao(scess_ctx *ctx, const double *ao_eri, const double *C, const double *eps,
                        int64_t nao, int64_t nmo, int64_t nocc, int32_t precision,
                        double *e_mp2);

/* ---- Spin-orbital cross-check solvers (CC.h:45-85).  The reference keeps
 * them to test the closed-shell solvers; they hold (2 nmo)^4 integrals and,
 * for (T), three o^3 v^3 spin-orbital tensors (o = 2 nocc, v = 2 nvirt).
 *
 * Spin-orbital CCSD (CCSD.cpp:21-106) or, with diis != 0, CCSD_DIIS
 * (CCSD-DIIS.cpp:17-198) from the CHEMISTS' MO integrals mo_eri(p,q,r,s) =
 * (pq|rs) (nmo^4, column-major, occupied first) and the canonical orbital
 * energies eps (nmo): <pq||rs> over 2 nmo spin orbitals (p = 2 x spatial +
 * spin; AntisymmetriseIntegrateOutSpinClosedShell, IntegralTransforms.cpp:
 * 135-162), t2 guess <ij||ab> / D_ijab, energy convergence 1e-6 within 50
 * iterations, DIIS over 6 vectors from iteration 3.  With triples != 0 and a
 * converged solve, result->E_T is the triples correction of CCSD_T
 * (CCSD_T.cpp:18-66).  t1_out (o x v) and t2_out (o x o x v x v) receive the
 * final amplitudes; g_out ((2 nmo)^4, may be NULL) the antisymmetrised
 * integrals (CCSD_Wfn::mints).  result: E_CCSD (0 unless converged, as the
 * reference's empty CCSD_Wfn), E_T, converged, iterations, last_dE; the
 * remaining fields are zero. */
int scess_ccsd_so_solve(scess_ctx *ctx, const double *mo_eri, const double *eps, int64_t nmo,
                        int64_t nocc, int32_t diis, int32_t triples, double *t1_out,
                        double *t2_out, double *g_out, scess_rccsd_result *result);

/* CalculateTriplesCorrection (CCSD_T.cpp:89-229) from the antisymmetrised
 * spin-orbital integrals g ((2 nmo)^4, as scess_ccsd_so_solve's g_out), the
 * spatial orbital energies eps (nmo) and spin-orbital t1, t2.  FP64. */
int scess_ccsd_so_triples(scess_ctx *ctx, const double *g, const double *eps, int64_t nmo,
                          int64_t nocc, const double *t1, const double *t2, double *e_t);

/* scess_einsum's FP64 contraction for callers that cannot allocate device
 * memory.  No counterpart in the reference.  Some host programs own every byte
 * of the GPU: a framework whose caching allocator has reserved the device's
 * memory, or an application that hands out a fixed arena at start-up and
 * forbids allocations later, because cudaMalloc and cudaFree can synchronise
 * the device and fail once that memory is spoken for.  This entry point
 * allocates nothing and needs no context: A, B and C are the caller's DEVICE
 * buffers (dense, column-major, extents as for scess_einsum), and the work is
 * queued on `stream` (a cudaStream_t; NULL is the default stream) of the
 * current device.  It returns once the work is queued; C is ready when the
 * stream reaches that point.
 *
 * Its scratch (the contraction's offset tables and split-K partial sums) is
 * one 16 MiB array inside this library, which every GPU that loads the
 * library holds until the process exits.  The tables need 16 (M + N + K)
 * bytes, M, N and K being the products of the extents of A's free labels, B's
 * free labels and the summed labels; a contraction with M + N + K above
 * 1,048,576 returns SCESS_ERR_TOO_LARGE and queues nothing.  Split-K uses what
 * the tables leave, with fewer splits (down to none) when that is too small.
 * Every call uses the same array and leaves its contents behind: calls whose
 * work overlaps on the GPU (other streams, other host threads) race on it, so
 * order them on one stream.  No part of it needs to start at zero: a call
 * writes all the scratch it reads before reading it.  The first call on a
 * device looks up the array's device address on that device (the CUDA runtime
 * loads the library's device code there), and so does the first call after
 * the device's CUDA context has changed (a cudaDeviceReset); make those calls
 * before any stream capture.  Returns SCESS_ERR_INVALID for a bad spec,
 * extents or null pointers, or when A, B or C is not device (or managed)
 * memory of the current device, SCESS_ERR_CUDA for a failed launch. */
int scess_einsum_static(const char *spec, double alpha, const double *A, int32_t a_nd,
                        const int64_t *a_ext, const double *B, int32_t b_nd,
                        const int64_t *b_ext, double beta, double *C, int32_t c_nd,
                        const int64_t *c_ext, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SCESS_CC_H */
