// Spin-orbital CCSD, CCSD-DIIS and (T): the reference's cross-check solvers
// (CCSD.cpp, CCSD-DIIS.cpp, CCSD_T.cpp) as FP64 engine einsums over views of
// the device-resident <pq||rs>.  The Fock matrix of canonical orbitals is
// diagonal (TransformFockToMO, CCSD.cpp:108-123 keeps only the diagonal), so
// the reference's F_ov terms are zero and the diagonal enters through the
// denominators alone.
#include <cfloat>
#include <cmath>
#include <deque>
#include <vector>

#include "ccsd_so.h"

namespace scess {

namespace {

unsigned grid_of(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 8 * kNumSMs));
}

// g(p,q,r,s) = chem(P,R,Q,S) [p~r][q~s] - chem(P,S,Q,R) [p~s][q~r], P = p/2,
// ~ = same spin (p % 2); the masks multiply as in the reference (:148-157).
__global__ void antisym_spin_kernel(int64_t n, const double *__restrict__ chem,
                                    double *__restrict__ g) {
  const int64_t N = 2 * n, total = N * N * N * N;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = x % N, q = (x / N) % N, r = (x / (N * N)) % N, s = x / (N * N * N);
    const double cm = (double)(((p & 1) == (r & 1)) && ((q & 1) == (s & 1)));
    const double xm = (double)(((p & 1) == (s & 1)) && ((q & 1) == (r & 1)));
    const int64_t P = p >> 1, Q = q >> 1, R = r >> 1, S = s >> 1;
    g[x] = chem[P + n * (R + n * (Q + n * S))] * cm - chem[P + n * (S + n * (Q + n * R))] * xm;
  }
}

// out(i,j,a,b) = s2 t2(i,j,a,b) + s1 t1(i,a) t1(j,b) [- s1 t1(i,b) t1(j,a)]:
// the tau and tilde-tau of CCSD.cpp:165-189 (anti) and the t2/2 + t1 t1
// intermediate of Wmbej (:341-343).
__global__ void so_tau_kernel(int64_t o, int64_t v, const double *__restrict__ t1,
                              const double *__restrict__ t2, double s2, double s1, int anti,
                              double *__restrict__ out) {
  const int64_t total = o * o * v * v;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = x % o, j = (x / o) % o, a = (x / (o * o)) % v, b = x / (o * o * v);
    double y = s2 * t2[x] + s1 * (t1[i + o * a] * t1[j + o * b]);
    if (anti) y -= s1 * (t1[i + o * b] * t1[j + o * a]);
    out[x] = y;
  }
}

// t(i,j,k,a,b,c) /= f_i + f_j + f_k - f_a - f_b - f_c, spin-orbital energies
// f_p = eps[p / 2] (MakeDijkabc, CCSD_T.cpp:128-148).
__global__ void so_triples_denom_kernel(int64_t o, int64_t v, const double *__restrict__ eps,
                                        double *__restrict__ t) {
  const int64_t total = o * o * o * v * v * v;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total;
       x += (int64_t)gridDim.x * blockDim.x) {
    int64_t y = x;
    const int64_t i = y % o; y /= o;
    const int64_t j = y % o; y /= o;
    const int64_t k = y % o; y /= o;
    const int64_t a = y % v; y /= v;
    const int64_t b = y % v;
    const int64_t c = y / v;
    const double d = eps[i >> 1] + eps[j >> 1] + eps[k >> 1] - eps[(o + a) >> 1] -
                     eps[(o + b) >> 1] - eps[(o + c) >> 1];
    t[x] /= d;
  }
}

// Spin-orbital energies f_p = eps[p / 2] (TransformFockToMO).
__global__ void spin_eps_kernel(int64_t N, const double *__restrict__ eps, double *__restrict__ f) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < N) f[p] = eps[p >> 1];
}

TV view4(const double *base, int64_t off, int64_t e0, int64_t e1, int64_t e2, int64_t e3,
         int64_t s0, int64_t s1, int64_t s2, int64_t s3) {
  TV t;
  t.p = const_cast<double *>(base) + off;
  t.nd = 4;
  const int64_t e[4] = {e0, e1, e2, e3}, s[4] = {s0, s1, s2, s3};
  for (int d = 0; d < 4; d++) {
    t.ext[d] = e[d];
    t.str[d] = s[d];
  }
  return t;
}

// Views of <pq||rs> (p + N q + N^2 r + N^3 s) over occupied (O) / virtual (V)
// ranges, e.g. sl("OOVV").
struct SoInts {
  const double *g;
  int64_t N, o, v;
  TV sl(const char *r) const {
    int64_t off = 0, e[4], st[4], stride = 1;
    for (int d = 0; d < 4; d++) {
      const bool occ = r[d] == 'O';
      off += (occ ? 0 : o) * stride;
      e[d] = occ ? o : v;
      st[d] = stride;
      stride *= N;
    }
    return view4(g, off, e[0], e[1], e[2], e[3], st[0], st[1], st[2], st[3]);
  }
};

// Solves the DIIS system with Eigen's PartialPivLU semantics (row pivoting on
// the largest magnitude in the column), CCSD-DIIS.cpp:151-153.
std::vector<double> partial_piv_lu_solve(std::vector<double> A, std::vector<double> b, int n) {
  auto at = [&](int i, int j) -> double & { return A[(size_t)i * n + j]; };
  for (int k = 0; k < n; k++) {
    int piv = k;
    for (int i = k + 1; i < n; i++)
      if (std::fabs(at(i, k)) > std::fabs(at(piv, k))) piv = i;
    if (piv != k) {
      for (int j = 0; j < n; j++) std::swap(at(k, j), at(piv, j));
      std::swap(b[k], b[piv]);
    }
    if (at(k, k) == 0.0) continue;
    for (int i = k + 1; i < n; i++) {
      const double l = at(i, k) / at(k, k);
      at(i, k) = l;
      for (int j = k + 1; j < n; j++) at(i, j) -= l * at(k, j);
      b[i] -= l * b[k];
    }
  }
  std::vector<double> x(n, 0.0);
  for (int i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (int j = i + 1; j < n; j++) s -= at(i, j) * x[j];
    x[i] = s / at(i, i);
  }
  return x;
}

// IterateCCSD work arrays.
struct SoWork {
  DTensor tau, ttau, tmp, Fae, Fmi, Fme, xvv, xoo, Wmnij, Wabef, Wmbej, Poooo, Pvvvv, P, X, r;
  SoWork(int64_t o, int64_t v)
      : tau({o, o, v, v}), ttau({o, o, v, v}), tmp({o, o, v, v}), Fae({v, v}), Fmi({o, o}),
        Fme({o, v}), xvv({v, v}), xoo({o, o}), Wmnij({o, o, o, o}), Wabef({v, v, v, v}),
        Wmbej({o, v, v, o}), Poooo({o, o, o, o}), Pvvvv({v, v, v, v}), P({o, o, v, v}),
        X({o, v, o, o}), r({o * v + o * o * v * v}) {}
};

void tau_of(Ctx &ctx, int64_t o, int64_t v, const double *t1, const double *t2, double s2,
            double s1, bool anti, double *out) {
  so_tau_kernel<<<grid_of(o * o * v * v), 256, 0, ctx.stream>>>(o, v, t1, t2, s2, s1, anti ? 1 : 0,
                                                                 out);
  SCESS_CHECK_LAUNCH();
}

// IterateCCSD, CCSD.cpp:161-480: amp = [t1 | t2] (column major) is replaced
// by the updated amplitudes.
void so_iterate(Ctx &ctx, const SoInts &I, const double *d_f, double *amp, SoWork &w) {
  const int64_t o = I.o, v = I.v;
  double *t1p = amp, *t2p = amp + o * v;
  const TV t1 = cm(t1p, {o, v}), t2 = cm(t2p, {o, o, v, v});
  const TV oovv = I.sl("OOVV"), ovvv = I.sl("OVVV"), ooov = I.sl("OOOV");
  tau_of(ctx, o, v, t1p, t2p, 1.0, 0.5, true, w.ttau.p());                 // :165-176
  tau_of(ctx, o, v, t1p, t2p, 1.0, 1.0, true, w.tau.p());                  // :178-189
  // Fae                                                                       :191-217
  einsum(ctx, "mf,mafe->ae", 1.0, t1, ovvv, 0.0, w.Fae.v);
  einsum(ctx, "mnaf,mnef->ae", -0.5, w.ttau.v, oovv, 1.0, w.Fae.v);
  // Fmi                                                                       :219-248
  einsum(ctx, "ne,mnie->mi", 1.0, t1, ooov, 0.0, w.Fmi.v);
  einsum(ctx, "inef,mnef->mi", 0.5, w.ttau.v, oovv, 1.0, w.Fmi.v);
  // Fme                                                                       :250-261
  einsum(ctx, "nf,mnef->me", 1.0, t1, oovv, 0.0, w.Fme.v);
  // Wmnij                                                                     :263-290
  permute(ctx, "mnij->mnij", 1.0, I.sl("OOOO"), 0.0, w.Wmnij.v);
  einsum(ctx, "je,mnie->mnij", 1.0, t1, ooov, 0.0, w.Poooo.v);
  permute(ctx, "mnij->mnij", 1.0, w.Poooo.v, 1.0, w.Wmnij.v);
  permute(ctx, "mnji->mnij", -1.0, w.Poooo.v, 1.0, w.Wmnij.v);
  einsum(ctx, "ijef,mnef->mnij", 0.25, w.tau.v, oovv, 1.0, w.Wmnij.v);
  // Wabef                                                                     :292-317
  permute(ctx, "abef->abef", 1.0, I.sl("VVVV"), 0.0, w.Wabef.v);
  einsum(ctx, "mb,amef->abef", 1.0, t1, I.sl("VOVV"), 0.0, w.Pvvvv.v);
  permute(ctx, "abef->abef", -1.0, w.Pvvvv.v, 1.0, w.Wabef.v);
  permute(ctx, "baef->abef", 1.0, w.Pvvvv.v, 1.0, w.Wabef.v);
  einsum(ctx, "mnab,mnef->abef", 0.25, w.tau.v, oovv, 1.0, w.Wabef.v);
  // Wmbej                                                                     :319-350
  permute(ctx, "mbej->mbej", 1.0, I.sl("OVVO"), 0.0, w.Wmbej.v);
  einsum(ctx, "jf,mbef->mbej", 1.0, t1, ovvv, 1.0, w.Wmbej.v);
  einsum(ctx, "nb,mnej->mbej", -1.0, t1, I.sl("OOVO"), 1.0, w.Wmbej.v);
  tau_of(ctx, o, v, t1p, t2p, 0.5, 1.0, false, w.tmp.p());               // t2/2 + t1(j,f) t1(n,b)
  einsum(ctx, "jnfb,mnef->mbej", -1.0, w.tmp.v, oovv, 1.0, w.Wmbej.v);

  double *r1p = w.r.p(), *r2p = w.r.p() + o * v;
  const TV r1 = cm(r1p, {o, v}), r2 = cm(r2p, {o, o, v, v});
  // t1 right-hand side                                                        :369-402
  einsum(ctx, "ie,ae->ia", 1.0, t1, w.Fae.v, 0.0, r1);
  einsum(ctx, "ma,mi->ia", -1.0, t1, w.Fmi.v, 1.0, r1);
  einsum(ctx, "imae,me->ia", 1.0, t2, w.Fme.v, 1.0, r1);
  einsum(ctx, "nf,naif->ia", -1.0, t1, I.sl("OVOV"), 1.0, r1);
  einsum(ctx, "imef,maef->ia", -0.5, t2, ovvv, 1.0, r1);
  einsum(ctx, "mnae,nmei->ia", -0.5, t2, I.sl("OOVO"), 1.0, r1);
  // t2 right-hand side                                                        :410-476
  permute(ctx, "ijab->ijab", 1.0, oovv, 0.0, r2);
  permute(ctx, "be->be", 1.0, w.Fae.v, 0.0, w.xvv.v);
  einsum(ctx, "mb,me->be", -0.5, t1, w.Fme.v, 1.0, w.xvv.v);
  einsum(ctx, "ijae,be->ijab", 1.0, t2, w.xvv.v, 0.0, w.P.v);
  permute(ctx, "ijab->ijab", 1.0, w.P.v, 1.0, r2);
  permute(ctx, "ijba->ijab", -1.0, w.P.v, 1.0, r2);
  permute(ctx, "mj->mj", 1.0, w.Fmi.v, 0.0, w.xoo.v);
  einsum(ctx, "me,je->mj", 0.5, w.Fme.v, t1, 1.0, w.xoo.v);
  einsum(ctx, "imab,mj->ijab", 1.0, t2, w.xoo.v, 0.0, w.P.v);
  permute(ctx, "ijab->ijab", -1.0, w.P.v, 1.0, r2);
  permute(ctx, "jiab->ijab", 1.0, w.P.v, 1.0, r2);
  einsum(ctx, "mnij,mnab->ijab", 0.5, w.Wmnij.v, w.tau.v, 1.0, r2);
  einsum(ctx, "ijef,abef->ijab", 0.5, w.tau.v, w.Wabef.v, 1.0, r2);
  einsum(ctx, "imae,mbej->ijab", 1.0, t2, w.Wmbej.v, 0.0, w.P.v);
  einsum(ctx, "mbej,ie->mbji", 1.0, I.sl("OVVO"), t1, 0.0, w.X.v);
  einsum(ctx, "mbji,ma->ijab", -1.0, w.X.v, t1, 1.0, w.P.v);
  permute(ctx, "ijab->ijab", 1.0, w.P.v, 1.0, r2);
  permute(ctx, "ijba->ijab", -1.0, w.P.v, 1.0, r2);
  permute(ctx, "jiab->ijab", -1.0, w.P.v, 1.0, r2);
  permute(ctx, "jiba->ijab", 1.0, w.P.v, 1.0, r2);
  einsum(ctx, "abej,ie->ijab", 1.0, I.sl("VVVO"), t1, 0.0, w.P.v);
  permute(ctx, "ijab->ijab", 1.0, w.P.v, 1.0, r2);
  permute(ctx, "jiab->ijab", -1.0, w.P.v, 1.0, r2);
  einsum(ctx, "mbij,ma->ijab", 1.0, I.sl("OVOO"), t1, 0.0, w.P.v);
  permute(ctx, "ijab->ijab", -1.0, w.P.v, 1.0, r2);
  permute(ctx, "ijba->ijab", 1.0, w.P.v, 1.0, r2);
  divide_denominators(o, v, d_f, r1p, r2p, t1p, t2p, ctx.stream);            // :478-479
}

// CalculateEnergyCCSD, CCSD.cpp:482-509: 1/4 <ij||ab> t2 + 1/2 <ij||ab> t1 t1.
double so_energy(Ctx &ctx, const DTensor &goovv, const double *amp, int64_t o, int64_t v,
                 DTensor &x) {
  cudaStream_t s = ctx.stream;
  einsum(ctx, "ijab,ia->jb", 1.0, goovv.v, cm(const_cast<double *>(amp), {o, v}), 0.0, x.v);
  dot(o * o * v * v, goovv.p(), amp + o * v, ctx.partials, ctx.dscalars, s);
  dot(o * v, x.p(), amp, ctx.partials, ctx.dscalars + 1, s);
  SCESS_CUDA(cudaMemcpyAsync(ctx.hscalars, ctx.dscalars, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  ctx.sync();
  return 0.25 * ctx.hscalars[0] + 0.5 * ctx.hscalars[1];
}

}  // namespace

void so_antisymmetrise(Ctx &ctx, const double *d_chem, int64_t n, double *d_g) {
  const int64_t N = 2 * n;
  antisym_spin_kernel<<<grid_of(N * N * N * N), 256, 0, ctx.stream>>>(n, d_chem, d_g);
  SCESS_CHECK_LAUNCH();
}

SoResult so_ccsd(Ctx &ctx, const double *d_g, const double *d_eps, int64_t nmo, int64_t nocc,
                 bool diis, bool triples, const Control &ctl, double *d_t1, double *d_t2) {
  constexpr double kConv = 1.0e-6;  // CCSD.cpp:24, CCSD-DIIS.cpp:20
  constexpr int kMaxIter = 50;      // CCSD.cpp:26, CCSD-DIIS.cpp:22
  constexpr int kMaxDiis = 6;       // CCSD-DIIS.cpp:25
  constexpr int kDiisStart = 3;     // CCSD-DIIS.cpp:119
  const int64_t N = 2 * nmo, o = 2 * nocc, v = N - o;
  const int64_t n1 = o * v, n2 = o * o * v * v, n = n1 + n2;
  cudaStream_t s = ctx.stream;
  const SoInts I{d_g, N, o, v};

  DTensor f({N});
  spin_eps_kernel<<<(unsigned)ceil_div(N, 256), 256, 0, s>>>(N, d_eps, f.p());
  SCESS_CHECK_LAUNCH();
  DTensor goovv({o, o, v, v}), xe({o, v}), amp({n}), prev({n});
  permute(ctx, "ijab->ijab", 1.0, I.sl("OOVV"), 0.0, goovv.v);
  // t1 = 0, t2 = <ij||ab> / D_ijab (CreateInitialT2Tensor, CCSD.cpp:150-157)
  DTensor zero({n1});
  SCESS_CUDA(cudaMemsetAsync(zero.p(), 0, n1 * sizeof(double), s));
  divide_denominators(o, v, f.p(), zero.p(), goovv.p(), amp.p(), amp.p() + n1, s);
  SCESS_CUDA(cudaMemsetAsync(amp.p(), 0, n1 * sizeof(double), s));
  SoWork w(o, v);

  // DIIS subspace (CCSD-DIIS.cpp:73-80): amplitudes and errors, oldest first
  const int slots = kMaxDiis + 1;
  DevMem vamp, verr, vptr, vcoef;
  std::deque<int> order;
  std::vector<std::vector<double>> gram;
  if (diis) {
    vamp.alloc((size_t)slots * n * sizeof(double));
    verr.alloc((size_t)slots * n * sizeof(double));
    vptr.alloc(slots * sizeof(double *));
    vcoef.alloc(slots * sizeof(double));
  }

  SoResult res;
  double E_last = DBL_MAX, E = 0.0;
  for (int it = 0; it < kMaxIter; it++) {
    ctl.poll();
    SCESS_CUDA(cudaMemcpyAsync(prev.p(), amp.p(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    so_iterate(ctx, I, f.p(), amp.p(), w);
    if (diis) {
      // error = updated - input; the stored vector becomes the updated
      // amplitudes (CCSD-DIIS.cpp:90-116)
      std::vector<bool> used(slots, false);
      for (int q : order) used[q] = true;
      int slot = 0;
      while (used[slot]) slot++;
      double *va = vamp.d() + (size_t)slot * n, *ve = verr.d() + (size_t)slot * n;
      SCESS_CUDA(cudaMemcpyAsync(va, amp.p(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      SCESS_CUDA(cudaMemcpyAsync(ve, amp.p(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      axpby(n, -1.0, prev.p(), 1.0, ve, s);
      order.push_back(slot);
      const int m = (int)order.size();
      for (int q = 0; q < m; q++)
        dot(n, verr.d() + (size_t)order[q] * n, ve, ctx.partials, ctx.dscalars + q, s);
      SCESS_CUDA(cudaMemcpyAsync(ctx.hscalars, ctx.dscalars, m * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
      ctx.sync();
      for (int q = 0; q < m - 1; q++) gram[q].push_back(ctx.hscalars[q]);
      gram.emplace_back(ctx.hscalars, ctx.hscalars + m);
      if (it >= kDiisStart) {                                                      // :119-166
        if ((int)order.size() > kMaxDiis) {
          order.pop_front();
          gram.erase(gram.begin());
          for (auto &row : gram) row.erase(row.begin());
        }
        const int k = (int)order.size();
        std::vector<double> B((size_t)(k + 1) * (k + 1), -1.0), rhs(k + 1, 0.0);
        B[(size_t)k * (k + 1) + k] = 0.0;
        double mx = 0.0;
        for (int i = 0; i < k; i++)
          for (int j = 0; j < k; j++) {
            B[(size_t)i * (k + 1) + j] = gram[i][j];
            mx = std::max(mx, std::fabs(gram[i][j]));
          }
        if (mx > 0.0)
          for (int i = 0; i < k; i++)
            for (int j = 0; j < k; j++) B[(size_t)i * (k + 1) + j] /= mx;
        rhs[k] = -1.0;
        std::vector<double> c = partial_piv_lu_solve(B, rhs, k + 1);
        c.resize(k);
        std::vector<const double *> hp(k);
        for (int q = 0; q < k; q++) hp[q] = vamp.d() + (size_t)order[q] * n;
        SCESS_CUDA(cudaMemcpyAsync(vptr.as<void>(), hp.data(), k * sizeof(double *),
                                   cudaMemcpyHostToDevice, s));
        SCESS_CUDA(cudaMemcpyAsync(vcoef.d(), c.data(), k * sizeof(double), cudaMemcpyHostToDevice, s));
        linear_combination(n, k, vptr.as<const double *>(), vcoef.d(), amp.p(), s);
        ctx.sync();  // hp / c are host buffers of this scope
      }
    }
    E = so_energy(ctx, goovv, amp.p(), o, v, xe);                                  // :161-165
    if (!std::isfinite(E)) throw Error(SCESS_ERR_INVALID, "non-finite CCSD energy (diverging amplitudes)");
    const double dE = std::fabs(E - E_last);
    ctx.logf(1, "   CCSD(%d): E(corr) = %.12g      dE = %.12g", it, E, dE);
    res.iterations = it + 1;
    res.last_E = E;
    res.last_dE = dE;
    if (dE < kConv) {
      res.converged = true;
      break;
    }
    E_last = E;
  }
  res.E_CCSD = res.converged ? E : 0.0;
  SCESS_CUDA(cudaMemcpyAsync(d_t1, amp.p(), n1 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SCESS_CUDA(cudaMemcpyAsync(d_t2, amp.p() + n1, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (triples && res.converged) res.E_T = so_triples(ctx, d_g, d_eps, nmo, nocc, d_t1, d_t2, ctl);
  ctx.sync();
  return res;
}

double so_triples(Ctx &ctx, const double *d_g, const double *d_eps, int64_t nmo, int64_t nocc,
                  const double *d_t1, const double *d_t2, const Control &ctl) {
  const int64_t N = 2 * nmo, o = 2 * nocc, v = N - o;
  cudaStream_t s = ctx.stream;
  const SoInts I{d_g, N, o, v};
  const TV t1 = cm(const_cast<double *>(d_t1), {o, v});
  const TV t2 = cm(const_cast<double *>(d_t2), {o, o, v, v});
  auto six = [&](DTensor &t) { return t.v; };
  DTensor A({o, o, o, v, v, v}), X({o, o, o, v, v, v}), T({o, o, o, v, v, v});
  ctl.poll();
  // t(ijkabc) = P(a/bc) P(k/ij) g_dkbc t_ijad - P(c/ab) P(i/jk) g_jklc t_ilab     :166-187
  einsum(ctx, "dkbc,ijad->ijkabc", 1.0, I.sl("VOVV"), t2, 0.0, six(A));
  permute(ctx, "ijkabc->ijkabc", 1.0, six(A), 0.0, six(X));                 // P(k/ij)
  permute(ctx, "kjiabc->ijkabc", -1.0, six(A), 1.0, six(X));
  permute(ctx, "ikjabc->ijkabc", -1.0, six(A), 1.0, six(X));
  permute(ctx, "ijkabc->ijkabc", 1.0, six(X), 0.0, six(T));                 // P(a/bc)
  permute(ctx, "ijkbac->ijkabc", -1.0, six(X), 1.0, six(T));
  permute(ctx, "ijkcba->ijkabc", -1.0, six(X), 1.0, six(T));
  einsum(ctx, "jklc,ilab->ijkabc", 1.0, I.sl("OOOV"), t2, 0.0, six(A));
  permute(ctx, "ijkabc->ijkabc", 1.0, six(A), 0.0, six(X));                 // P(i/jk)
  permute(ctx, "jikabc->ijkabc", -1.0, six(A), 1.0, six(X));
  permute(ctx, "kjiabc->ijkabc", -1.0, six(A), 1.0, six(X));
  permute(ctx, "ijkabc->ijkabc", -1.0, six(X), 1.0, six(T));                // -= P(c/ab)
  permute(ctx, "ijkcba->ijkabc", 1.0, six(X), 1.0, six(T));
  permute(ctx, "ijkacb->ijkabc", 1.0, six(X), 1.0, six(T));
  so_triples_denom_kernel<<<grid_of(o * o * o * v * v * v), 256, 0, s>>>(o, v, d_eps, T.p());
  SCESS_CHECK_LAUNCH();
  ctl.poll();
  // D_ijab t_ijab^(3) = 1/2 P(ab) g_efbm t_ijmaef - 1/2 P(ij) g_jemn t_imnabe    :190-206
  DTensor x({o, o, v, v}), vt3({o, o, v, v}), y({o, v});
  einsum(ctx, "efbm,ijmaef->ijab", 1.0, I.sl("VVVO"), six(T), 0.0, x.v);
  permute(ctx, "ijab->ijab", 0.5, x.v, 0.0, vt3.v);
  permute(ctx, "ijba->ijab", -0.5, x.v, 1.0, vt3.v);
  einsum(ctx, "jemn,imnabe->ijab", 1.0, I.sl("OVOO"), six(T), 0.0, x.v);
  permute(ctx, "ijab->ijab", -0.5, x.v, 1.0, vt3.v);
  permute(ctx, "jiab->ijab", 0.5, x.v, 1.0, vt3.v);
  // E[4] = 1/4 t2 . (D t3), E[5] = 1/4 t1 . (g_bcjk t_ijkabc)                   :208-227
  einsum(ctx, "bcjk,ijkabc->ia", 1.0, I.sl("VVOO"), six(T), 0.0, y.v);
  dot(o * o * v * v, d_t2, vt3.p(), ctx.partials, ctx.dscalars, s);
  dot(o * v, y.p(), d_t1, ctx.partials, ctx.dscalars + 1, s);
  SCESS_CUDA(cudaMemcpyAsync(ctx.hscalars, ctx.dscalars, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  ctx.sync();
  return 0.25 * ctx.hscalars[0] + 0.25 * ctx.hscalars[1];
}

}  // namespace scess
