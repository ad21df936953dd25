// Hand-written reverse-mode adjoint (vector-Jacobian products) of the engine's
// recorded forward ops, and the CCSD residual VJP built on it.
#pragma once
#include <vector>

#include "engine.h"
#include "rccsd.h"

namespace scess {

// Maps forward tensors (by allocation range) to their gradient buffers, so that
// a strided view of a forward tensor has a gradient view with the same strides.
class GradMap {
 public:
  void add(const double *base, int64_t n, double *grad);
  // Gradient view of `t`; false when the tensor is not tracked (a constant).
  bool grad_of(const TV &t, TV &g) const;

 private:
  struct Entry {
    const double *base;
    int64_t n;
    double *g;
  };
  std::vector<Entry> e_;
};

// Reverse sweep over the tape: for every op, accumulate the cotangent of its
// output into its inputs' gradients (einsum: gA += alpha gC.B, gB += alpha A.gC;
// permute: gX += alpha P^-1 gY; tau: gt2 += gtau, gt1 += gtau.t1 (both
// pairings); PlusTranspose: gX += gOut + gOut^T), then scale the output's
// gradient by beta (zero for an overwrite).  `be` chooses the contraction
// backend of the adjoint einsums (FP64 or tensor cores).
void reverse_sweep(Ctx &ctx, const Tape &tape, const GradMap &gm, Backend be);

// VJP of the CCSD residual numerators R(t1, t2; eri) (rccsd_residual) for
// cotangents gR = [gR1 | gR2]: gAmp = [gT1 | gT2], and, when g_eri is not
// null, the integral gradient in eri layout (nmo^4).
void rccsd_residual_vjp(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc,
                        const double *d_amp, const double *d_gR, Backend fwd, Backend adj,
                        double *d_gAmp, double *d_geri);

}  // namespace scess

namespace scess {

// Lambda equations and unrelaxed one-particle density (no counterpart in the
// reference).  Omega(t; f) = R(t) + the Fock terms that UpdateAmplitudes
// drops for canonical orbitals (RCCSD.cpp:13-15, :109); at f = diag(eps) they
// equal -D t.  With E(t; f) = 2 sum f_ia t_ia + sum L_oovv tau and the
// Lagrangian L = E + lambda . Omega, the Lambda equations are
// dE/dt + (dOmega/dt)^T lambda = 0 on the closed-shell subspace
// t2(ijab) = t2(jiba) (solved by lambda += (dE/dt + J^T lambda)/D with the t2
// part of J^T lambda symmetrised, plus DIIS), and gamma_pq = dL/df_pq.
struct LambdaResult {
  int converged = 0, iterations = 0;
  double last_rms = 0.0;
};
LambdaResult rccsd_lambda(Ctx &ctx, const double *d_eri, const double *eps_host, int64_t nmo,
                          int64_t nocc, const double *d_amp, const scess_rccsd_options &opts,
                          Backend be, const Control &ctl, double *d_lambda);
// gamma (nmo x nmo, column-major, symmetric) into d_dm1.
void rccsd_rdm1(Ctx &ctx, const double *d_eri, const double *eps_host, int64_t nmo, int64_t nocc,
                const double *d_amp, const double *d_lambda, Backend be, double *d_dm1);

}  // namespace scess
