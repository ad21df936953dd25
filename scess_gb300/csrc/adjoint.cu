// Reverse sweep over recorded forward ops and the CCSD residual VJP.
//
// The reference has no derivative code; this is a new capability.  Every
// forward op of the residual is an einsum, a permutation, tau = t2 + t1 t1 or
// the final PlusTranspose, and the adjoint of each is again one of those ops
// on the same GPU engine, so the VJP runs at the forward's speed with either
// backend.
#include <cmath>
#include <deque>
#include <memory>
#include <string>

#include "adjoint.h"
#include "kernels.h"

namespace scess {

void GradMap::add(const double *base, int64_t n, double *grad) { e_.push_back({base, n, grad}); }

bool GradMap::grad_of(const TV &t, TV &g) const {
  for (const Entry &x : e_) {
    if (t.p >= x.base && t.p < x.base + x.n) {
      g = t;
      g.p = x.g + (t.p - x.base);
      return true;
    }
  }
  return false;
}

namespace {

void split_spec(const std::string &s, std::string &a, std::string &b, std::string &c) {
  const size_t arrow = s.find("->");
  const std::string lhs = s.substr(0, arrow);
  c = s.substr(arrow + 2);
  const size_t comma = lhs.find(',');
  if (comma == std::string::npos) {
    a = lhs;
    b.clear();
  } else {
    a = lhs.substr(0, comma);
    b = lhs.substr(comma + 1);
  }
}

// Y *= beta over the view (beta = 0 clears it).
void scale_view(Ctx &ctx, const TV &Y, double beta) {
  if (beta == 1.0) return;
  PermDesc d;
  d.nd = Y.nd;
  for (int k = 0; k < Y.nd; k++) {
    d.ext[k] = Y.ext[k];
    d.xs[k] = Y.str[k];
    d.ys[k] = Y.str[k];
  }
  permute_add(d, 0.0, Y.p, beta, Y.p, ctx.stream);
}

}  // namespace

void reverse_sweep(Ctx &ctx, const Tape &tape, const GradMap &gm, Backend be) {
  Tape *saved = ctx.tape;
  ctx.tape = nullptr;  // the adjoint ops are not recorded
  for (auto it = tape.ops.rbegin(); it != tape.ops.rend(); ++it) {
    const TapeOp &op = *it;
    TV gC;
    if (!gm.grad_of(op.C, gC)) continue;
    switch (op.kind) {
      case TapeOp::EINSUM: {
        std::string a, b, c;
        split_spec(op.spec, a, b, c);
        TV gA, gB;
        if (gm.grad_of(op.A, gA)) {
          const std::string s = c + "," + b + "->" + a;  // gA += alpha gC . B
          einsum(ctx, s.c_str(), op.alpha, gC, op.B, 1.0, gA, be);
        }
        if (gm.grad_of(op.B, gB)) {
          const std::string s = a + "," + c + "->" + b;  // gB += alpha A . gC
          einsum(ctx, s.c_str(), op.alpha, op.A, gC, 1.0, gB, be);
        }
        scale_view(ctx, gC, op.beta);
        break;
      }
      case TapeOp::PERMUTE: {
        std::string a, b, c;
        split_spec(op.spec, a, b, c);
        TV gX;
        if (gm.grad_of(op.A, gX)) {
          const std::string s = c + "->" + a;  // gX += alpha P^-1 gY
          permute(ctx, s.c_str(), op.alpha, gC, 1.0, gX);
        }
        scale_view(ctx, gC, op.beta);
        break;
      }
      case TapeOp::TAU: {  // tau = t2 + t1 (x) t1
        TV gt1, gt2;
        if (gm.grad_of(op.B, gt2)) permute(ctx, "ijab->ijab", 1.0, gC, 1.0, gt2);
        if (gm.grad_of(op.A, gt1)) {
          einsum(ctx, "ijab,jb->ia", 1.0, gC, op.A, 1.0, gt1, Backend::FP64);
          einsum(ctx, "jiba,jb->ia", 1.0, gC, op.A, 1.0, gt1, Backend::FP64);
        }
        scale_view(ctx, gC, 0.0);
        break;
      }
      case TapeOp::PLUS_T: {  // out += X + X^T
        TV gX;
        if (gm.grad_of(op.A, gX)) plus_transpose(op.o, op.v, 1.0, gC.p, gX.p, ctx.stream);
        break;
      }
    }
  }
  ctx.tape = saved;
}

void rccsd_residual_vjp(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc,
                        const double *d_amp, const double *d_gR, Backend fwd, Backend adj,
                        double *d_gAmp, double *d_geri) {
  const int64_t o = nocc, v = nmo - nocc, N = nmo;
  const int64_t n = o * v + o * o * v * v;
  cudaStream_t s = ctx.stream;
  Tape tape;
  ctx.tape = &tape;
  RccsdBlocks B;
  RccsdWork w;
  DTensor R({n});
  try {
    B.build(ctx, d_eri, nmo, nocc);
    w.alloc(o, v, fwd == Backend::FP64);
    rccsd_residual(ctx, B, d_amp, nullptr, fwd, w, R.p());
  } catch (...) {
    ctx.tape = nullptr;
    throw;
  }
  ctx.tape = nullptr;

  GradMap gm;
  std::vector<std::unique_ptr<DTensor>> gbuf;
  auto track = [&](const DTensor &t) {
    if (!t.p()) return;
    auto g = std::make_unique<DTensor>();
    g->mem.alloc((size_t)t.size() * sizeof(double));
    g->v = t.v;
    g->v.p = g->mem.d();
    SCESS_CUDA(cudaMemsetAsync(g->p(), 0, (size_t)t.size() * sizeof(double), s));
    gm.add(t.p(), t.size(), g->p());
    gbuf.push_back(std::move(g));
  };
  for (const DTensor *t : {&w.tau, &w.Foo, &w.Fvv, &w.Fov, &w.Fovt1, &w.Loo, &w.Lvv, &w.X,
                           &w.tmp_abic, &w.tmp_kibj, &w.tmp_akij, &w.Woooo, &w.Wvvvv, &w.Wvoov, &w.Wvovo,
                           &w.tmp_lkci, &w.tmp_lcki, &w.Yd, &B.L_oovv, &B.L_ovov})
    track(*t);
  SCESS_CUDA(cudaMemsetAsync(d_gAmp, 0, (size_t)n * sizeof(double), s));
  gm.add(d_amp, n, d_gAmp);
  DTensor gR({n});
  SCESS_CUDA(cudaMemcpyAsync(gR.p(), d_gR, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  gm.add(R.p(), n, gR.p());
  if (d_geri) {
    SCESS_CUDA(cudaMemsetAsync(d_geri, 0, (size_t)N * N * N * N * sizeof(double), s));
    gm.add(d_eri, N * N * N * N, d_geri);
  }
  reverse_sweep(ctx, tape, gm, adj);
  ctx.sync();
}

}  // namespace scess

// ---------------------------------------------------------------------------------------------
// Lambda equations and the unrelaxed one-particle density.

namespace scess {

namespace {

// l_out = l + (dE + g) / D with D_ia = e_i - e_a, D_ijab = D_ia + D_jb.  The
// closed-shell doubles are constrained to t2(ijab) = t2(jiba), so only the
// symmetric part of the t2 gradient enters (its antisymmetric part is not a
// stationarity condition and the iteration is unstable on it).
__global__ void lambda_step_kernel(int64_t o, int64_t v, const double *__restrict__ eps,
                                   const double *__restrict__ l, const double *__restrict__ dE,
                                   const double *__restrict__ g, double *__restrict__ out) {
  const int64_t n1 = o * v, n2 = o * o * v * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n1 + n2;
       e += (int64_t)gridDim.x * blockDim.x) {
    double d;
    if (e < n1) {
      const int64_t i = e % o, a = e / o;
      d = eps[i] - eps[o + a];
    } else {
      const int64_t x = e - n1;
      const int64_t i = x % o, j = (x / o) % o, a = (x / (o * o)) % v, b = x / (o * o * v);
      d = (eps[i] - eps[o + a]) + (eps[j] - eps[o + b]);
      const int64_t xt = j + o * i + o * o * b + o * o * v * a;
      out[e] = l[e] + (dE[e] + 0.5 * (g[e] + g[n1 + xt])) / d;
      continue;
    }
    out[e] = l[e] + (dE[e] + g[e]) / d;
  }
}

// gamma from dL/df: symmetric halves of the oo and vv blocks, ov = vo = (g_fov + 2 t1) / 2.
__global__ void rdm_assemble_kernel(int64_t o, int64_t v, const double *__restrict__ goo,
                                    const double *__restrict__ gvv, const double *__restrict__ gov,
                                    const double *__restrict__ t1, double *__restrict__ dm) {
  const int64_t N = o + v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < N * N;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e % N, q = e / N;
    double val;
    if (p < o && q < o) val = 0.5 * (goo[p + o * q] + goo[q + o * p]);
    else if (p >= o && q >= o) val = 0.5 * (gvv[(p - o) + v * (q - o)] + gvv[(q - o) + v * (p - o)]);
    else if (p < o) val = 0.5 * (gov[p + o * (q - o)] + 2.0 * t1[p + o * (q - o)]);
    else val = 0.5 * (gov[q + o * (p - o)] + 2.0 * t1[q + o * (p - o)]);
    dm[e] = val;
  }
}

__global__ void diag_kernel(int64_t n, const double *__restrict__ e, double *__restrict__ M) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * n;
       i += (int64_t)gridDim.x * blockDim.x)
    M[i] = (i % n == i / n) ? e[i % n] : 0.0;
}

unsigned blocks_for(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 8 * kNumSMs));
}

// Forward Omega(t; f) at f = diag(eps) recorded on a tape, with gradient buffers
// for every tensor the reverse sweep reaches.
struct Lagrangian {
  int64_t o = 0, v = 0, N = 0, n = 0;
  RccsdBlocks B;
  RccsdWork w;
  DTensor R, foo, fvv, fov, tmpF, lvvF, looF, X2F, eps;
  Tape tape;
  GradMap gm;
  std::vector<std::unique_ptr<DTensor>> gbuf;
  DTensor gR;
  double *g_foo = nullptr, *g_fvv = nullptr, *g_fov = nullptr;

  void build(Ctx &ctx, const double *d_eri, const double *eps_host, int64_t nmo, int64_t nocc,
             const double *d_amp, double *d_gAmp, Backend be) {
    o = nocc;
    v = nmo - nocc;
    N = nmo;
    n = o * v + o * o * v * v;
    cudaStream_t s = ctx.stream;
    eps = DTensor({N});
    upload(ctx, eps.p(), eps_host, N);
    foo = DTensor({o, o});
    fvv = DTensor({v, v});
    fov = DTensor({o, v});
    diag_kernel<<<blocks_for(o * o), 256, 0, s>>>(o, eps.p(), foo.p());
    SCESS_CHECK_LAUNCH();
    diag_kernel<<<blocks_for(v * v), 256, 0, s>>>(v, eps.p() + o, fvv.p());
    SCESS_CHECK_LAUNCH();
    SCESS_CUDA(cudaMemsetAsync(fov.p(), 0, fov.size() * sizeof(double), s));
    tmpF = DTensor({o, o});
    lvvF = DTensor({v, v});
    looF = DTensor({o, o});
    X2F = DTensor({o, o, v, v});
    R = DTensor({n});
    ctx.tape = &tape;
    try {
      B.build(ctx, d_eri, nmo, nocc);
      w.alloc(o, v, be == Backend::FP64);
      rccsd_residual(ctx, B, d_amp, nullptr, be, w, R.p());
      // Fock terms of the general closed-shell equations
      const TV t1 = cm(const_cast<double *>(d_amp), {o, v});
      const TV t2 = cm(const_cast<double *>(d_amp) + o * v, {o, o, v, v});
      const TV R1 = cm(R.p(), {o, v}), R2 = cm(R.p() + o * v, {o, o, v, v});
      einsum(ctx, "ac,ic->ia", 1.0, fvv.v, t1, 1.0, R1);
      einsum(ctx, "ki,ka->ia", -1.0, foo.v, t1, 1.0, R1);
      einsum(ctx, "kc,kica->ia", 2.0, fov.v, t2, 1.0, R1);
      einsum(ctx, "kc,ikca->ia", -1.0, fov.v, t2, 1.0, R1);
      einsum(ctx, "kc,ic->ki", 1.0, fov.v, t1, 0.0, tmpF.v);
      einsum(ctx, "ki,ka->ia", -1.0, tmpF.v, t1, 1.0, R1);
      permute(ctx, "ia->ia", 1.0, fov.v, 1.0, R1);
      permute(ctx, "ac->ac", 1.0, fvv.v, 0.0, lvvF.v);
      einsum(ctx, "kc,ka->ac", -1.0, fov.v, t1, 1.0, lvvF.v);
      permute(ctx, "ki->ki", 1.0, foo.v, 0.0, looF.v);
      permute(ctx, "ki->ki", 1.0, tmpF.v, 1.0, looF.v);
      einsum(ctx, "ac,ijcb->ijab", 1.0, lvvF.v, t2, 0.0, X2F.v);
      einsum(ctx, "ki,kjab->ijab", -1.0, looF.v, t2, 1.0, X2F.v);
      plus_transpose(o, v, 1.0, X2F.p(), R2.p, s);
      TapeOp op;
      op.kind = TapeOp::PLUS_T;
      op.A = X2F.v;
      op.C = R2;
      op.o = o;
      op.v = v;
      tape.ops.push_back(op);
    } catch (...) {
      ctx.tape = nullptr;
      throw;
    }
    ctx.tape = nullptr;
    auto track = [&](const DTensor &t) -> double * {
      if (!t.p()) return nullptr;
      auto g = std::make_unique<DTensor>();
      g->mem.alloc((size_t)t.size() * sizeof(double));
      g->v = t.v;
      g->v.p = g->mem.d();
      gm.add(t.p(), t.size(), g->p());
      double *ptr = g->p();
      gbuf.push_back(std::move(g));
      return ptr;
    };
    for (const DTensor *t : {&w.tau, &w.Foo, &w.Fvv, &w.Fov, &w.Fovt1, &w.Loo, &w.Lvv, &w.X,
                             &w.tmp_abic, &w.tmp_kibj, &w.tmp_akij, &w.Woooo, &w.Wvvvv, &w.Wvoov, &w.Wvovo,
                             &w.tmp_lkci, &w.tmp_lcki, &w.Yd, &tmpF, &lvvF, &looF, &X2F})
      track(*t);
    g_foo = track(foo);
    g_fvv = track(fvv);
    g_fov = track(fov);
    gm.add(d_amp, n, d_gAmp);
    gR = DTensor({n});
    gm.add(R.p(), n, gR.p());
    amp_grad_ = d_gAmp;
  }

  // d_gAmp = (dOmega/dt)^T seed; the Fock gradients land in g_foo, g_fvv, g_fov.
  void vjp(Ctx &ctx, const double *d_seed, Backend be) {
    cudaStream_t s = ctx.stream;
    for (auto &g : gbuf) SCESS_CUDA(cudaMemsetAsync(g->p(), 0, g->size() * sizeof(double), s));
    SCESS_CUDA(cudaMemsetAsync(amp_grad_, 0, (size_t)n * sizeof(double), s));
    SCESS_CUDA(cudaMemcpyAsync(gR.p(), d_seed, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    reverse_sweep(ctx, tape, gm, be);
  }

 private:
  double *amp_grad_ = nullptr;
};

}  // namespace

LambdaResult rccsd_lambda(Ctx &ctx, const double *d_eri, const double *eps_host, int64_t nmo,
                          int64_t nocc, const double *d_amp, const scess_rccsd_options &opts,
                          Backend be, const Control &ctl, double *d_lambda) {
  const int64_t o = nocc, v = nmo - nocc, n1 = o * v, n2 = o * o * v * v, n = n1 + n2;
  cudaStream_t s = ctx.stream;
  DTensor gAmp({n});
  Lagrangian lag;
  lag.build(ctx, d_eri, eps_host, nmo, nocc, d_amp, gAmp.p(), be);
  // dE/dt: dE/dt1 = sum_jb L(i,j,a,b) t1(j,b) + L(j,i,b,a) t1(j,b), dE/dt2 = L_oovv
  DTensor dE({n});
  const TV t1 = cm(const_cast<double *>(d_amp), {o, v});
  einsum(ctx, "ijab,jb->ia", 1.0, lag.B.L_oovv.v, t1, 0.0, cm(dE.p(), {o, v}));
  einsum(ctx, "jiba,jb->ia", 1.0, lag.B.L_oovv.v, t1, 1.0, cm(dE.p(), {o, v}));
  SCESS_CUDA(cudaMemcpyAsync(dE.p() + n1, lag.B.L_oovv.p(), n2 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // start: lambda = dE / D
  DTensor zero({n}), lnew({n});
  SCESS_CUDA(cudaMemsetAsync(zero.p(), 0, n * sizeof(double), s));
  lambda_step_kernel<<<blocks_for(n), 256, 0, s>>>(o, v, lag.eps.p(), zero.p(), dE.p(), zero.p(), d_lambda);
  SCESS_CHECK_LAUNCH();

  const int maxv = std::max(1, opts.max_diis_vectors);
  DevMem dv((size_t)maxv * n * sizeof(double)), de((size_t)maxv * n * sizeof(double));
  DevMem vecptr((size_t)maxv * sizeof(double *)), coefd((size_t)maxv * sizeof(double));
  std::deque<int> order;
  std::vector<std::vector<double>> gram;
  LambdaResult res;
  for (int it = 0; it < opts.max_iterations; it++) {
    ctl.poll();
    lag.vjp(ctx, d_lambda, be);
    lambda_step_kernel<<<blocks_for(n), 256, 0, s>>>(o, v, lag.eps.p(), d_lambda, dE.p(), gAmp.p(), lnew.p());
    SCESS_CHECK_LAUNCH();
    int slot;
    if ((int)order.size() < maxv) {
      slot = (int)order.size();
    } else {
      slot = order.front();
      order.pop_front();
      gram.erase(gram.begin());
      for (auto &row : gram) row.erase(row.begin());
    }
    double *va = dv.d() + (size_t)slot * n, *ve = de.d() + (size_t)slot * n;
    SCESS_CUDA(cudaMemcpyAsync(va, lnew.p(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SCESS_CUDA(cudaMemcpyAsync(ve, lnew.p(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    axpby(n, -1.0, d_lambda, 1.0, ve, s);
    order.push_back(slot);
    const int nv = (int)order.size();
    for (int q = 0; q < nv; q++)
      dot(n, de.d() + (size_t)order[q] * n, ve, ctx.partials, ctx.dscalars + q, s);
    SCESS_CUDA(cudaMemcpyAsync(ctx.hscalars, ctx.dscalars, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
    ctx.sync();
    for (int q = 0; q < nv - 1; q++) gram[q].push_back(ctx.hscalars[q]);
    gram.emplace_back(ctx.hscalars, ctx.hscalars + nv);
    const double rms = std::sqrt(ctx.hscalars[nv - 1] / (double)n);
    if (it >= opts.diis_start) {
      std::vector<double> c = diis_coefficients(gram);
      std::vector<const double *> hp(nv);
      for (int q = 0; q < nv; q++) hp[q] = dv.d() + (size_t)order[q] * n;
      SCESS_CUDA(cudaMemcpyAsync(vecptr.as<void>(), hp.data(), nv * sizeof(double *), cudaMemcpyHostToDevice, s));
      SCESS_CUDA(cudaMemcpyAsync(coefd.d(), c.data(), nv * sizeof(double), cudaMemcpyHostToDevice, s));
      linear_combination(n, nv, vecptr.as<const double *>(), coefd.d(), d_lambda, s);
      ctx.sync();
    } else {
      SCESS_CUDA(cudaMemcpyAsync(d_lambda, lnew.p(), n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    ctx.logf(1, "   Lambda(%d): rms(dl) = %.12g", it, rms);
    res.iterations = it + 1;
    res.last_rms = rms;
    if (rms < opts.amplitude_convergence) {
      res.converged = 1;
      break;
    }
  }
  ctx.sync();
  return res;
}

void rccsd_rdm1(Ctx &ctx, const double *d_eri, const double *eps_host, int64_t nmo, int64_t nocc,
                const double *d_amp, const double *d_lambda, Backend be, double *d_dm1) {
  const int64_t o = nocc, v = nmo - nocc, n = o * v + o * o * v * v;
  DTensor gAmp({n});
  Lagrangian lag;
  lag.build(ctx, d_eri, eps_host, nmo, nocc, d_amp, gAmp.p(), be);
  lag.vjp(ctx, d_lambda, be);
  rdm_assemble_kernel<<<blocks_for(nmo * nmo), 256, 0, ctx.stream>>>(o, v, lag.g_foo, lag.g_fvv,
                                                                     lag.g_fov, d_amp, d_dm1);
  SCESS_CHECK_LAUNCH();
  ctx.sync();
}

}  // namespace scess
