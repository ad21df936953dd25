// C ABI of the engine (include/scess_cc.h): argument checks, host<->device
// transfers and exception-to-status translation around the C++ drivers.
#include <memory>
#include <vector>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>

#include "adjoint.h"
#include "ccsd_so.h"
#include "gemm_tc.h"
#include "rccsd.h"
#include "triples.h"

struct scess_ctx {
  scess::Ctx *impl = nullptr;
  std::string err;
};

struct scess_rccsd_state {
  scess_ctx *ctx = nullptr;
  scess::RccsdState *impl = nullptr;
};

namespace {

using scess::Error;

template <class F>
int guard(scess_ctx *ctx, F &&f) {
  if (!ctx || !ctx->impl) return SCESS_ERR_INVALID;
  int code = SCESS_OK;
  scess::CurrentCtx cur(ctx->impl);  // device blocks released during the call are cached
  try {
    SCESS_CUDA(cudaSetDevice(ctx->impl->device));
    f(*ctx->impl);
    ctx->err.clear();
  } catch (const Error &e) {
    ctx->err = e.what();
    code = e.code;
  } catch (const std::bad_alloc &) {
    ctx->err = "host allocation failed";
    code = SCESS_ERR_OOM;
  } catch (const std::exception &e) {
    ctx->err = e.what();
    code = SCESS_ERR_CUDA;
  }
  // Packings cached during a plain call are keyed by device pointers of that call.
  cudaStreamSynchronize(ctx->impl->stream);
  if (ctx->impl->tc) ctx->impl->tc->clear_cache(nullptr);
  if (code != SCESS_OK) cudaGetLastError();
  return code;
}

void check_shape(int64_t nmo, int64_t nocc) {
  if (nmo <= 0 || nocc <= 0 || nocc >= nmo)
    throw Error(SCESS_ERR_INVALID, "need 0 < nocc < nmo");
  if (nmo > 4096) throw Error(SCESS_ERR_INVALID, "nmo too large");
}

void need(const void *p, const char *what) {
  if (!p) throw Error(SCESS_ERR_INVALID, std::string("null pointer: ") + what);
}

void host_finite(const double *x, int64_t n, const char *what) {
  for (int64_t i = 0; i < n; i++)
    if (!std::isfinite(x[i])) throw Error(SCESS_ERR_INVALID, std::string("non-finite value in ") + what);
}

void device_finite(scess::Ctx &ctx, const double *x, int64_t n, const char *what) {
  int *flag = reinterpret_cast<int *>(ctx.dscalars + 63);
  SCESS_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx.stream));
  scess::check_finite(n, x, flag, ctx.stream);
  int h = 0;
  SCESS_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  if (h) throw Error(SCESS_ERR_INVALID, std::string("non-finite value in ") + what);
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// eri (nmo^4) on the device from the host eri, checked finite.  DF inputs never
// come here: their states contract the integral blocks they read from B.
scess::DTensor device_eri(scess::Ctx &ctx, const double *eri, int64_t N) {
  auto t0 = std::chrono::steady_clock::now();
  scess::DTensor d({N, N, N, N});
  ctx.timer.host("eri_alloc", ms_since(t0));
  t0 = std::chrono::steady_clock::now();
  scess::upload(ctx, d.p(), eri, N * N * N * N);
  ctx.timer.host("eri_upload", ms_since(t0));
  t0 = std::chrono::steady_clock::now();
  device_finite(ctx, d.p(), N * N * N * N, "eri");
  ctx.timer.host("eri_check", ms_since(t0));
  return d;
}

// DF factors B (naux x nmo x nmo) on the device, checked finite.
scess::DTensor device_B(scess::Ctx &ctx, const double *B, int64_t naux, int64_t N) {
  if (naux <= 0) throw Error(SCESS_ERR_INVALID, "bad naux");
  scess::DTensor dB({naux, N, N});
  scess::upload(ctx, dB.p(), B, naux * N * N);
  device_finite(ctx, dB.p(), naux * N * N, "B");
  return dB;
}

scess::RccsdState *make_state(scess::Ctx &c, const double *eri, const double *B, int64_t naux,
                              const double *eps, int64_t nmo, int64_t nocc,
                              const double *f12_residual, const double *f12_energy,
                              const scess_rccsd_options &o) {
  check_shape(nmo, nocc);
  need(eps, "eps");
  host_finite(eps, nmo, "eps");
  if (o.max_iterations < 0 || o.max_diis_vectors < 1 || o.diis_start < 0 ||
      (o.precision != SCESS_PRECISION_FP64 && o.precision != SCESS_PRECISION_MIXED))
    throw Error(SCESS_ERR_INVALID, "bad options");
  const int64_t v = nmo - nocc;
  if (f12_residual) host_finite(f12_residual, nocc * nocc * v * v, "f12_residual");
  if (f12_energy) host_finite(f12_energy, nocc * nocc * v * v, "f12_energy");
  scess::SolveInput in;
  in.eps_host = eps;
  in.f12_residual = f12_residual;
  in.f12_energy = f12_energy;
  scess::RccsdState *st = nullptr;
  if (B) {  // DF state: the integral blocks are contracted from B, no nmo^4 eri
    scess::DTensor dB = device_B(c, B, naux, nmo);
    const auto t0 = std::chrono::steady_clock::now();
    st = new scess::RccsdState(c, std::move(dB), naux, nmo, nocc, in, o);
    c.sync();
    c.timer.host("state_build", ms_since(t0));
    return st;
  }
  scess::DTensor d_eri = device_eri(c, eri, nmo);
  const auto t0 = std::chrono::steady_clock::now();
  st = new scess::RccsdState(c, std::move(d_eri), nmo, nocc, in, o);
  c.sync();
  c.timer.host("state_build", ms_since(t0));
  return st;
}

int solve_common(scess_ctx *ctx, const double *eri, const double *B, int64_t naux,
                 const double *eps, int64_t nmo, int64_t nocc, const double *f12_residual,
                 const double *f12_energy, const scess_rccsd_options *opts, double *t1_out,
                 double *t2_out, scess_rccsd_result *result) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(eps, "eps");
    need(t1_out, "t1_out");
    need(t2_out, "t2_out");
    need(result, "result");
    host_finite(eps, nmo, "eps");
    scess_rccsd_options o;
    if (opts) o = *opts;
    else scess_rccsd_default_options(&o);
    if (o.max_iterations < 0 || o.max_diis_vectors < 1 || o.diis_start < 0 ||
        (o.precision != SCESS_PRECISION_FP64 && o.precision != SCESS_PRECISION_MIXED))
      throw Error(SCESS_ERR_INVALID, "bad options");
    const int64_t v = nmo - nocc;
    if (f12_residual) host_finite(f12_residual, nocc * nocc * v * v, "f12_residual");
    if (f12_energy) host_finite(f12_energy, nocc * nocc * v * v, "f12_energy");
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    ctl.time_limit_s = o.time_limit_s;
    scess::SolveInput in;
    in.eps_host = eps;
    in.f12_residual = f12_residual;
    in.f12_energy = f12_energy;
    std::unique_ptr<scess::RccsdState> stp;
    if (B)  // DF: the integral blocks are contracted from B, no nmo^4 eri
      stp.reset(new scess::RccsdState(c, device_B(c, B, naux, nmo), naux, nmo, nocc, in, o));
    else
      stp.reset(new scess::RccsdState(c, device_eri(c, eri, nmo), nmo, nocc, in, o));
    ctl.poll();
    scess::RccsdState &st = *stp;
    if (o.resume) st.set_amplitudes(t1_out, t2_out);
    else st.mp2_guess();
    scess::rccsd_solve(c, st, ctl, t1_out, t2_out, result);
  });
}

}  // namespace

extern "C" {

int64_t scess_launch_count(void) { return (int64_t)scess::g_launches.load(); }

const char *scess_status_string(int status) {
  switch (status) {
    case SCESS_OK: return "ok";
    case SCESS_ERR_INVALID: return "invalid argument";
    case SCESS_ERR_OOM: return "out of memory";
    case SCESS_ERR_CUDA: return "CUDA error";
    case SCESS_ERR_CANCELLED: return "cancelled";
    case SCESS_ERR_TIMEOUT: return "time limit exceeded";
    case SCESS_ERR_UNSUPPORTED: return "unsupported";
    case SCESS_ERR_TOO_LARGE: return "too large for the fixed scratch";
    default: return "unknown status";
  }
}

int scess_ctx_create(int device, scess_ctx **out) {
  if (!out) return SCESS_ERR_INVALID;
  *out = nullptr;
  try {
    auto *c = new scess_ctx;
    try {
      c->impl = new scess::Ctx(device);
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
    return SCESS_OK;
  } catch (const Error &e) {
    return e.code;
  } catch (const std::bad_alloc &) {
    return SCESS_ERR_OOM;
  } catch (...) {
    return SCESS_ERR_CUDA;
  }
}

void scess_ctx_destroy(scess_ctx *ctx) {
  if (!ctx) return;
  if (ctx->impl) {
    cudaSetDevice(ctx->impl->device);
    delete ctx->impl;
  }
  delete ctx;
}

const char *scess_ctx_last_error(const scess_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

int scess_ctx_set_memory_limit(scess_ctx *ctx, int64_t bytes) {
  if (!ctx || !ctx->impl || bytes < 0) return SCESS_ERR_INVALID;
  ctx->impl->mem_limit = (size_t)bytes;
  return SCESS_OK;
}

int64_t scess_ctx_memory_held(const scess_ctx *ctx) {
  return (ctx && ctx->impl) ? (int64_t)ctx->impl->mem_held : -1;
}

int scess_ctx_arm_wait_expiry(scess_ctx *ctx, int64_t wait_cycles) {
  if (wait_cycles < (int64_t(1) << 16) || wait_cycles > (int64_t(1) << 40)) return SCESS_ERR_INVALID;
  return guard(ctx, [&](scess::Ctx &c) { c.tensor_cores().arm_wait_expiry(wait_cycles); });
}

int scess_ctx_set_callbacks(scess_ctx *ctx, scess_cancel_fn cancel, scess_log_fn log, void *user) {
  if (!ctx || !ctx->impl) return SCESS_ERR_INVALID;
  ctx->impl->cancel = cancel;
  ctx->impl->log = log;
  ctx->impl->user = user;
  return SCESS_OK;
}

void scess_rccsd_default_options(scess_rccsd_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->energy_convergence = 1.0e-10;   // RCCSD.cpp:302
  o->amplitude_convergence = 1.0e-8; // :303
  o->max_iterations = 100;           // :304
  o->diis_start = 2;                 // :306
  o->max_diis_vectors = 8;           // :307
  o->precision = SCESS_PRECISION_FP64;
  o->refine_sweeps = 2;
  o->mixed_energy_switch = 1.0e-8;
  o->mixed_amplitude_switch = 1.0e-6;
}

int scess_rccsd_solve(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                      int64_t nocc, const double *f12_residual, const double *f12_energy,
                      const scess_rccsd_options *opts, double *t1_out, double *t2_out,
                      scess_rccsd_result *result) {
  if (!eri) return SCESS_ERR_INVALID;
  return solve_common(ctx, eri, nullptr, 0, eps, nmo, nocc, f12_residual, f12_energy, opts,
                      t1_out, t2_out, result);
}

int scess_rccsd_solve_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                         int64_t nmo, int64_t nocc, const double *f12_residual,
                         const double *f12_energy, const scess_rccsd_options *opts,
                         double *t1_out, double *t2_out, scess_rccsd_result *result) {
  if (!B || naux <= 0) return SCESS_ERR_INVALID;
  return solve_common(ctx, nullptr, B, naux, eps, nmo, nocc, f12_residual, f12_energy, opts,
                      t1_out, t2_out, result);
}

static int triples_common(scess_ctx *ctx, const double *eri, const double *B, int64_t naux,
                          const double *eps, int64_t nmo, int64_t nocc, const double *t1,
                          const double *t2, int32_t precision, double *e_t) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(eps, "eps");
    need(t1, "t1");
    need(t2, "t2");
    need(e_t, "e_t");
    if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
      throw Error(SCESS_ERR_INVALID, "bad precision");
    const int64_t o = nocc, v = nmo - nocc;
    host_finite(eps, nmo, "eps");
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    // DF input: (T) reads only (ia|bf), (ia|mj) and (ia|jb), formed from B on
    // the device; the nmo^4 eri is not built
    scess::DTensor d_eri, dB;
    if (eri) {
      d_eri = device_eri(c, eri, nmo);
    } else {
      dB = scess::DTensor({naux, nmo, nmo});
      scess::upload(c, dB.p(), B, naux * nmo * nmo);
      device_finite(c, dB.p(), naux * nmo * nmo, "B");
    }
    scess::DTensor d_eps({nmo}), d_t1({o, v}), d_t2({o, o, v, v});
    scess::upload(c, d_eps.p(), eps, nmo);
    scess::upload(c, d_t1.p(), t1, o * v);
    scess::upload(c, d_t2.p(), t2, o * o * v * v);
    device_finite(c, d_t1.p(), o * v, "t1");
    device_finite(c, d_t2.p(), o * o * v * v, "t2");
    ctl.poll();
    *e_t = scess::rccsd_triples(c, d_eri.p(), nmo, nocc, d_eps.p(), d_t1.p(), d_t2.p(),
                                precision == SCESS_PRECISION_MIXED, ctl, nullptr, dB.p(), naux);
  });
}

int scess_rccsd_triples(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                        int64_t nocc, const double *t1, const double *t2, int32_t precision,
                        double *e_t) {
  if (!eri) return SCESS_ERR_INVALID;
  return triples_common(ctx, eri, nullptr, 0, eps, nmo, nocc, t1, t2, precision, e_t);
}

int scess_rccsd_triples_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                           int64_t nmo, int64_t nocc, const double *t1, const double *t2,
                           int32_t precision, double *e_t) {
  if (!B || naux <= 0) return SCESS_ERR_INVALID;
  return triples_common(ctx, nullptr, B, naux, eps, nmo, nocc, t1, t2, precision, e_t);
}

static int triples_vjp_common(scess_ctx *ctx, const double *eri, const double *B, int64_t naux,
                              const double *eps, int64_t nmo, int64_t nocc, const double *t1,
                              const double *t2, int32_t precision, double g_e, double *e_t,
                              double *g_t1, double *g_t2, double *g_eri, double *g_B) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
      throw Error(SCESS_ERR_INVALID, "bad precision");
    need(eps, "eps");
    need(t1, "t1");
    need(t2, "t2");
    need(g_t1, "g_t1");
    need(g_t2, "g_t2");
    if (!std::isfinite(g_e)) throw Error(SCESS_ERR_INVALID, "g_e is not finite");
    const int64_t o = nocc, v = nmo - nocc, N = nmo, n1 = o * v, n2 = o * o * v * v;
    const int64_t N4 = N * N * N * N;
    host_finite(eps, nmo, "eps");
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    scess::DTensor d_eri({N, N, N, N}), dB;
    scess::Tape dfTape;
    if (eri) {
      scess::upload(c, d_eri.p(), eri, N4);
      device_finite(c, d_eri.p(), N4, "eri");
    } else {
      dB = scess::DTensor({naux, N, N});
      scess::upload(c, dB.p(), B, naux * N * N);
      device_finite(c, dB.p(), naux * N * N, "B");
      c.tape = &dfTape;  // eri(p,q,r,s) = sum_Q B(Q,p,r) B(Q,q,s), recorded for g_B
      scess::einsum(c, "Qpr,Qqs->pqrs", 1.0, dB.v, dB.v, 0.0, d_eri.v, scess::Backend::FP64);
      c.tape = nullptr;
    }
    scess::DTensor d_eps({nmo}), d_t1({o, v}), d_t2({o, o, v, v}), gt1({o, v}), gt2({o, o, v, v});
    scess::upload(c, d_eps.p(), eps, nmo);
    scess::upload(c, d_t1.p(), t1, n1);
    scess::upload(c, d_t2.p(), t2, n2);
    device_finite(c, d_t1.p(), n1, "t1");
    device_finite(c, d_t2.p(), n2, "t2");
    SCESS_CUDA(cudaMemsetAsync(gt1.p(), 0, n1 * sizeof(double), c.stream));
    SCESS_CUDA(cudaMemsetAsync(gt2.p(), 0, n2 * sizeof(double), c.stream));
    const bool need_eri = g_eri || g_B;
    scess::DTensor geri;
    if (need_eri) {
      geri = scess::DTensor({N, N, N, N});
      SCESS_CUDA(cudaMemsetAsync(geri.p(), 0, N4 * sizeof(double), c.stream));
    }
    ctl.poll();
    const double et = scess::rccsd_triples_vjp(c, d_eri.p(), nmo, nocc, d_eps.p(), d_t1.p(),
                                               d_t2.p(), g_e, ctl, gt1.p(), gt2.p(),
                                               need_eri ? geri.p() : nullptr,
                                               precision == SCESS_PRECISION_MIXED);
    if (e_t) *e_t = et;
    scess::download(c, g_t1, gt1.p(), n1);
    scess::download(c, g_t2, gt2.p(), n2);
    if (g_eri) scess::download(c, g_eri, geri.p(), N4);
    if (g_B) {
      scess::DTensor gB({naux, N, N});
      SCESS_CUDA(cudaMemsetAsync(gB.p(), 0, (size_t)naux * N * N * sizeof(double), c.stream));
      scess::GradMap gm;
      gm.add(d_eri.p(), N4, geri.p());
      gm.add(dB.p(), naux * N * N, gB.p());
      scess::reverse_sweep(c, dfTape, gm, scess::Backend::FP64);
      scess::download(c, g_B, gB.p(), naux * N * N);
    }
  });
}

int scess_rccsd_triples_vjp(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                            int64_t nocc, const double *t1, const double *t2, int32_t precision,
                            double g_e, double *e_t, double *g_t1, double *g_t2, double *g_eri) {
  if (!eri) return SCESS_ERR_INVALID;
  return triples_vjp_common(ctx, eri, nullptr, 0, eps, nmo, nocc, t1, t2, precision, g_e, e_t,
                            g_t1, g_t2, g_eri, nullptr);
}

int scess_rccsd_triples_vjp_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                               int64_t nmo, int64_t nocc, const double *t1, const double *t2,
                               int32_t precision, double g_e, double *e_t, double *g_t1,
                               double *g_t2, double *g_B) {
  if (!B || naux <= 0) return SCESS_ERR_INVALID;
  return triples_vjp_common(ctx, nullptr, B, naux, eps, nmo, nocc, t1, t2, precision, g_e, e_t,
                            g_t1, g_t2, nullptr, g_B);
}

static int state_create(scess_ctx *ctx, const double *eri, const double *B, int64_t naux,
                        const double *eps, int64_t nmo, int64_t nocc, const double *f12_residual,
                        const double *f12_energy, const scess_rccsd_options *opts,
                        scess_rccsd_state **out) {
  if (!out) return SCESS_ERR_INVALID;
  *out = nullptr;
  return guard(ctx, [&](scess::Ctx &c) {
    scess_rccsd_options o;
    if (opts) o = *opts;
    else scess_rccsd_default_options(&o);
    std::unique_ptr<scess::RccsdState> st(
        make_state(c, eri, B, naux, eps, nmo, nocc, f12_residual, f12_energy, o));
    const auto t0 = std::chrono::steady_clock::now();
    st->mp2_guess();
    c.sync();
    c.timer.host("mp2_guess", ms_since(t0));
    auto *h = new scess_rccsd_state;
    h->ctx = ctx;
    h->impl = st.release();
    *out = h;
  });
}

int scess_rccsd_state_create(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                             int64_t nocc, const double *f12_residual, const double *f12_energy,
                             const scess_rccsd_options *opts, scess_rccsd_state **out) {
  if (!eri) return SCESS_ERR_INVALID;
  return state_create(ctx, eri, nullptr, 0, eps, nmo, nocc, f12_residual, f12_energy, opts, out);
}

int scess_rccsd_state_create_df(scess_ctx *ctx, const double *B, int64_t naux, const double *eps,
                                int64_t nmo, int64_t nocc, const double *f12_residual,
                                const double *f12_energy, const scess_rccsd_options *opts,
                                scess_rccsd_state **out) {
  if (!B || naux <= 0) return SCESS_ERR_INVALID;
  return state_create(ctx, nullptr, B, naux, eps, nmo, nocc, f12_residual, f12_energy, opts, out);
}

void scess_rccsd_state_destroy(scess_rccsd_state *state) {
  if (!state) return;
  if (state->impl) {
    cudaSetDevice(state->ctx->impl->device);
    cudaStreamSynchronize(state->ctx->impl->stream);
    const auto t0 = std::chrono::steady_clock::now();
    scess::CurrentCtx cur(state->ctx->impl);  // the state's blocks go to its context's cache
    if (state->ctx->impl->tc) state->ctx->impl->tc->clear_cache(state->impl);
    delete state->impl;
    state->ctx->impl->timer.host("state_destroy", ms_since(t0));
  }
  delete state;
}

int scess_rccsd_state_iterate(scess_rccsd_state *state, int32_t n_iterations,
                              scess_rccsd_result *result, double *device_ms) {
  if (!state || !state->impl || n_iterations < 0) return SCESS_ERR_INVALID;
  return guard(state->ctx, [&](scess::Ctx &c) {
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    ctl.time_limit_s = state->impl->options().time_limit_s;
    if (c.tc) c.tc->set_cache_owner(state->impl);
    struct Reset {
      scess::Ctx &c;
      ~Reset() { if (c.tc) c.tc->set_cache_owner(nullptr); }
    } reset{c};
    c.tensor_cores().set_cache_owner(state->impl);
    state->impl->iterate(n_iterations, ctl);
    if (result) *result = state->impl->result();
    if (device_ms) *device_ms = state->impl->last_device_ms();
  });
}

int scess_rccsd_state_triples(scess_rccsd_state *state, int32_t precision, double *e_t,
                              double *device_ms) {
  if (!state || !state->impl || !e_t) return SCESS_ERR_INVALID;
  if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
    return SCESS_ERR_INVALID;
  return guard(state->ctx, [&](scess::Ctx &c) {
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    cudaEvent_t a, b;
    SCESS_CUDA(cudaEventCreate(&a));
    SCESS_CUDA(cudaEventCreate(&b));
    SCESS_CUDA(cudaEventRecord(a, c.stream));
    auto *st = state->impl;
    // a DF state's (T) contracts its integral slices from B
    *e_t = scess::rccsd_triples(c, st->d_eri(), st->nmo(), st->nocc(), st->d_eps(), st->d_t1(),
                                st->d_t2(), precision == SCESS_PRECISION_MIXED, ctl, nullptr,
                                st->d_B(), st->naux());
    SCESS_CUDA(cudaEventRecord(b, c.stream));
    SCESS_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    SCESS_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (device_ms) *device_ms = ms;
  });
}

int scess_rccsd_state_amplitudes(scess_rccsd_state *state, double *t1_out, double *t2_out) {
  if (!state || !state->impl) return SCESS_ERR_INVALID;
  return guard(state->ctx, [&](scess::Ctx &c) {
    const auto t0 = std::chrono::steady_clock::now();
    state->impl->get_amplitudes(t1_out, t2_out);
    c.timer.host("amplitudes_download", ms_since(t0));
  });
}

int scess_rccsd_state_set_amplitudes(scess_rccsd_state *state, const double *t1,
                                     const double *t2) {
  if (!state || !state->impl || !t1 || !t2) return SCESS_ERR_INVALID;
  return guard(state->ctx, [&](scess::Ctx &) { state->impl->set_amplitudes(t1, t2); });
}

int scess_ctx_profile(scess_ctx *ctx, int32_t enable) {
  return guard(ctx, [&](scess::Ctx &c) {
    c.timer.collect();
    if (enable) c.timer.agg.clear();
    c.timer.on = enable != 0;
  });
}

int scess_ctx_profile_report(scess_ctx *ctx, char *buf, int64_t buflen) {
  if (!buf || buflen <= 0) return SCESS_ERR_INVALID;
  return guard(ctx, [&](scess::Ctx &c) {
    c.timer.collect();
    std::string js = "{";
    bool first = true;
    for (auto &kv : c.timer.agg) {
      char tmp[512];
      snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f, \"flops\": %.6e, \"bytes\": %.6e}",
               first ? "" : ", ", kv.first.c_str(), (long long)kv.second.launches, kv.second.ms,
               kv.second.flops, kv.second.bytes);
      js += tmp;
      first = false;
    }
    js += "}";
    std::strncpy(buf, js.c_str(), (size_t)buflen - 1);
    buf[buflen - 1] = 0;
  });
}

static int residual_common(scess_ctx *ctx, const double *eri, const double *B, int64_t naux,
                           int64_t nmo, int64_t nocc, const double *t1, const double *t2,
                           const double *t2_driver, int32_t precision, double *r1_out,
                           double *r2_out) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(t1, "t1");
    need(t2, "t2");
    need(r1_out, "r1_out");
    need(r2_out, "r2_out");
    const int64_t o = nocc, v = nmo - nocc, n1 = o * v, n2 = o * o * v * v, N = nmo;
    scess::DTensor d_eri;
    if (eri) {
      d_eri = device_eri(c, eri, nmo);
    } else {
      // eri(p,q,r,s) = sum_Q B(Q,p,r) B(Q,q,s) in FP64, as the DF adjoint forms it
      scess::DTensor dB = device_B(c, B, naux, nmo);
      d_eri = scess::DTensor({N, N, N, N});
      scess::einsum(c, "Qpr,Qqs->pqrs", 1.0, dB.v, dB.v, 0.0, d_eri.v, scess::Backend::FP64);
    }
    scess::RccsdBlocks blocks;
    blocks.build(c, d_eri.p(), nmo, nocc);
    scess::DTensor amp({n1 + n2}), R({n1 + n2}), drv;
    scess::upload(c, amp.p(), t1, n1);
    scess::upload(c, amp.p() + n1, t2, n2);
    if (t2_driver) {
      drv = scess::DTensor({o, o, v, v});
      scess::upload(c, drv.p(), t2_driver, n2);
    }
    const bool mixed = precision == SCESS_PRECISION_MIXED;
    scess::RccsdWork w;
    w.alloc(o, v, !mixed);
    scess::rccsd_residual(c, blocks, amp.p(), drv.p(), mixed ? scess::Backend::MIXED : scess::Backend::FP64,
                          w, R.p());
    scess::download(c, r1_out, R.p(), n1);
    scess::download(c, r2_out, R.p() + n1, n2);
    if (mixed) c.tensor_cores().check_error();
  });
}

int scess_rccsd_residual(scess_ctx *ctx, const double *eri, int64_t nmo, int64_t nocc,
                         const double *t1, const double *t2, const double *t2_driver,
                         int32_t precision, double *r1_out, double *r2_out) {
  if (!eri) return SCESS_ERR_INVALID;
  return residual_common(ctx, eri, nullptr, 0, nmo, nocc, t1, t2, t2_driver, precision, r1_out,
                         r2_out);
}

int scess_rccsd_residual_df(scess_ctx *ctx, const double *B, int64_t naux, int64_t nmo,
                            int64_t nocc, const double *t1, const double *t2,
                            const double *t2_driver, int32_t precision, double *r1_out,
                            double *r2_out) {
  if (!B || naux <= 0) return SCESS_ERR_INVALID;
  return residual_common(ctx, nullptr, B, naux, nmo, nocc, t1, t2, t2_driver, precision, r1_out,
                         r2_out);
}

static int residual_vjp_common(scess_ctx *ctx, const double *eri, const double *B, int64_t naux,
                               int64_t nmo, int64_t nocc, const double *t1, const double *t2,
                               const double *g_r1, const double *g_r2, int32_t precision,
                               double *g_t1, double *g_t2, double *g_eri, double *g_B) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(t1, "t1");
    need(t2, "t2");
    need(g_r1, "g_r1");
    need(g_r2, "g_r2");
    need(g_t1, "g_t1");
    need(g_t2, "g_t2");
    if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
      throw Error(SCESS_ERR_INVALID, "bad precision");
    const int64_t o = nocc, v = nmo - nocc, N = nmo, n1 = o * v, n2 = o * o * v * v;
    const int64_t N4 = N * N * N * N;
    scess::DTensor d_eri({N, N, N, N}), dB;
    scess::Tape dfTape;
    if (eri) {
      scess::upload(c, d_eri.p(), eri, N4);
      device_finite(c, d_eri.p(), N4, "eri");
    } else {
      dB = scess::DTensor({naux, N, N});
      scess::upload(c, dB.p(), B, naux * N * N);
      device_finite(c, dB.p(), naux * N * N, "B");
      c.tape = &dfTape;  // eri(p,q,r,s) = sum_Q B(Q,p,r) B(Q,q,s), recorded for g_B
      scess::einsum(c, "Qpr,Qqs->pqrs", 1.0, dB.v, dB.v, 0.0, d_eri.v, scess::Backend::FP64);
      c.tape = nullptr;
    }
    scess::DTensor amp({n1 + n2}), gR({n1 + n2}), gAmp({n1 + n2}), geri;
    scess::upload(c, amp.p(), t1, n1);
    scess::upload(c, amp.p() + n1, t2, n2);
    scess::upload(c, gR.p(), g_r1, n1);
    scess::upload(c, gR.p() + n1, g_r2, n2);
    const bool need_eri = g_eri || g_B;
    if (need_eri) geri = scess::DTensor({N, N, N, N});
    const scess::Backend be =
        precision == SCESS_PRECISION_MIXED ? scess::Backend::MIXED : scess::Backend::FP64;
    scess::rccsd_residual_vjp(c, d_eri.p(), nmo, nocc, amp.p(), gR.p(), be, be, gAmp.p(),
                              need_eri ? geri.p() : nullptr);
    scess::download(c, g_t1, gAmp.p(), n1);
    scess::download(c, g_t2, gAmp.p() + n1, n2);
    if (g_eri) scess::download(c, g_eri, geri.p(), N4);
    if (g_B) {
      scess::DTensor gB({naux, N, N});
      SCESS_CUDA(cudaMemsetAsync(gB.p(), 0, (size_t)naux * N * N * sizeof(double), c.stream));
      scess::GradMap gm;
      gm.add(d_eri.p(), N4, geri.p());
      gm.add(dB.p(), naux * N * N, gB.p());
      scess::reverse_sweep(c, dfTape, gm, scess::Backend::FP64);
      scess::download(c, g_B, gB.p(), naux * N * N);
    }
    if (precision == SCESS_PRECISION_MIXED) c.tensor_cores().check_error();
  });
}

int scess_rccsd_residual_vjp(scess_ctx *ctx, const double *eri, int64_t nmo, int64_t nocc,
                             const double *t1, const double *t2, const double *g_r1,
                             const double *g_r2, int32_t precision, double *g_t1, double *g_t2,
                             double *g_eri) {
  if (!eri) return SCESS_ERR_INVALID;
  return residual_vjp_common(ctx, eri, nullptr, 0, nmo, nocc, t1, t2, g_r1, g_r2, precision, g_t1,
                             g_t2, g_eri, nullptr);
}

int scess_rccsd_residual_vjp_df(scess_ctx *ctx, const double *B, int64_t naux, int64_t nmo,
                                int64_t nocc, const double *t1, const double *t2,
                                const double *g_r1, const double *g_r2, int32_t precision,
                                double *g_t1, double *g_t2, double *g_B) {
  if (!B || naux <= 0) return SCESS_ERR_INVALID;
  return residual_vjp_common(ctx, nullptr, B, naux, nmo, nocc, t1, t2, g_r1, g_r2, precision, g_t1,
                             g_t2, nullptr, g_B);
}

int scess_rccsd_lambda(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                       int64_t nocc, const double *t1, const double *t2,
                       const scess_rccsd_options *opts, double *l1_out, double *l2_out,
                       scess_rccsd_result *result) {
  if (!eri) return SCESS_ERR_INVALID;
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(eps, "eps");
    need(t1, "t1");
    need(t2, "t2");
    need(l1_out, "l1_out");
    need(l2_out, "l2_out");
    host_finite(eps, nmo, "eps");
    scess_rccsd_options o;
    if (opts) o = *opts;
    else scess_rccsd_default_options(&o);
    const int64_t oc = nocc, v = nmo - nocc, n1 = oc * v, n2 = oc * oc * v * v;
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    ctl.time_limit_s = o.time_limit_s;
    scess::DTensor d_eri = device_eri(c, eri, nmo);
    scess::DTensor amp({n1 + n2}), lam({n1 + n2});
    scess::upload(c, amp.p(), t1, n1);
    scess::upload(c, amp.p() + n1, t2, n2);
    const scess::Backend be =
        o.precision == SCESS_PRECISION_MIXED ? scess::Backend::MIXED : scess::Backend::FP64;
    const scess::LambdaResult r =
        scess::rccsd_lambda(c, d_eri.p(), eps, nmo, nocc, amp.p(), o, be, ctl, lam.p());
    scess::download(c, l1_out, lam.p(), n1);
    scess::download(c, l2_out, lam.p() + n1, n2);
    if (result) {
      std::memset(result, 0, sizeof(*result));
      result->converged = r.converged;
      result->iterations = r.iterations;
      result->last_rms = r.last_rms;
    }
  });
}

int scess_rccsd_rdm1(scess_ctx *ctx, const double *eri, const double *eps, int64_t nmo,
                     int64_t nocc, const double *t1, const double *t2, const double *l1,
                     const double *l2, int32_t precision, double *dm1_out) {
  if (!eri) return SCESS_ERR_INVALID;
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(eps, "eps");
    need(t1, "t1");
    need(t2, "t2");
    need(l1, "l1");
    need(l2, "l2");
    need(dm1_out, "dm1_out");
    const int64_t oc = nocc, v = nmo - nocc, n1 = oc * v, n2 = oc * oc * v * v;
    scess::DTensor d_eri = device_eri(c, eri, nmo);
    scess::DTensor amp({n1 + n2}), lam({n1 + n2}), dm({nmo, nmo});
    scess::upload(c, amp.p(), t1, n1);
    scess::upload(c, amp.p() + n1, t2, n2);
    scess::upload(c, lam.p(), l1, n1);
    scess::upload(c, lam.p() + n1, l2, n2);
    scess::rccsd_rdm1(c, d_eri.p(), eps, nmo, nocc, amp.p(), lam.p(),
                      precision == SCESS_PRECISION_MIXED ? scess::Backend::MIXED
                                                         : scess::Backend::FP64,
                      dm.p());
    scess::download(c, dm1_out, dm.p(), nmo * nmo);
  });
}

int scess_einsum(scess_ctx *ctx, const char *spec, double alpha, const double *A, int32_t a_nd,
                 const int64_t *a_ext, const double *B, int32_t b_nd, const int64_t *b_ext,
                 double beta, double *C, int32_t c_nd, const int64_t *c_ext, int32_t precision) {
  return guard(ctx, [&](scess::Ctx &c) {
    need(spec, "spec");
    need(A, "A");
    need(B, "B");
    need(C, "C");
    auto mk = [&](int nd, const int64_t *ext, scess::DTensor &t) {
      if (nd < 1 || nd > 6 || !ext) throw Error(SCESS_ERR_INVALID, "bad rank");
      int64_t n = 1;
      for (int d = 0; d < nd; d++) {
        if (ext[d] <= 0) throw Error(SCESS_ERR_INVALID, "bad extent");
        n *= ext[d];
      }
      t.mem.alloc((size_t)n * sizeof(double));
      t.v.p = t.mem.d();
      t.v.nd = nd;
      int64_t s = 1;
      for (int d = 0; d < nd; d++) {
        t.v.ext[d] = ext[d];
        t.v.str[d] = s;
        s *= ext[d];
      }
      return n;
    };
    scess::DTensor dA, dB, dC;
    const int64_t na = mk(a_nd, a_ext, dA), nbb = mk(b_nd, b_ext, dB), nc = mk(c_nd, c_ext, dC);
    scess::upload(c, dA.p(), A, na);
    scess::upload(c, dB.p(), B, nbb);
    scess::upload(c, dC.p(), C, nc);
    scess::einsum(c, spec, alpha, dA.v, dB.v, beta, dC.v,
                  precision == SCESS_PRECISION_MIXED ? scess::Backend::TENSOR : scess::Backend::FP64);
    scess::download(c, C, dC.p(), nc);
    if (precision == SCESS_PRECISION_MIXED) c.tensor_cores().check_error();
  });
}

}  // extern "C"

extern "C" {

int scess_transform_tei(scess_ctx *ctx, const double *tei, int64_t nao, const double *A,
                        int64_t na, const double *B, int64_t nb, const double *C, int64_t nc,
                        const double *D, int64_t nd, int32_t chem_to_phys, int32_t precision,
                        double *out) {
  return guard(ctx, [&](scess::Ctx &c) {
    need(tei, "tei");
    need(A, "A");
    need(B, "B");
    need(C, "C");
    need(D, "D");
    need(out, "out");
    if (nao <= 0 || na <= 0 || nb <= 0 || nc <= 0 || nd <= 0)
      throw Error(SCESS_ERR_INVALID, "bad dimensions");
    if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
      throw Error(SCESS_ERR_INVALID, "bad precision");
    const scess::Backend be =
        precision == SCESS_PRECISION_MIXED ? scess::Backend::TENSOR : scess::Backend::FP64;
    const int64_t n = nao, n4 = n * n * n * n;
    auto mat = [&](const double *h, int64_t cols, const char *name) {
      scess::DTensor m({n, cols});
      scess::upload(c, m.p(), h, n * cols);
      device_finite(c, m.p(), n * cols, name);
      return m;
    };
    scess::DTensor dA = mat(A, na, "A"), dB = mat(B, nb, "B"), dC = mat(C, nc, "C"),
                   dD = mat(D, nd, "D");
    // IntegralTransforms.cpp:44-55: one index at a time, at most two 4-index tensors alive
    scess::DTensor x({n, n, n, n});
    scess::upload(c, x.p(), tei, n4);
    device_finite(c, x.p(), n4, "tei");
    scess::DTensor y({n, n, n, nd});
    scess::einsum(c, "mnkl,ls->mnks", 1.0, x.v, dD.v, 0.0, y.v, be);   // (mu nu|kap s)
    x = scess::DTensor({n, n, nc, nd});
    scess::einsum(c, "mnks,kr->mnrs", 1.0, y.v, dC.v, 0.0, x.v, be);   // (mu nu|r s)
    y = scess::DTensor({n, nb, nc, nd});
    scess::einsum(c, "mnrs,nq->mqrs", 1.0, x.v, dB.v, 0.0, y.v, be);   // (mu q|r s)
    x = scess::DTensor({na, nb, nc, nd});
    scess::einsum(c, "mqrs,mp->pqrs", 1.0, y.v, dA.v, 0.0, x.v, be);   // (p q|r s)
    if (chem_to_phys) {                                                // :57-59, pqrs -> prqs
      y = scess::DTensor({na, nc, nb, nd});
      scess::permute(c, "pqrs->prqs", 1.0, x.v, 0.0, y.v);
      scess::download(c, out, y.p(), na * nb * nc * nd);
    } else {
      scess::download(c, out, x.p(), na * nb * nc * nd);
    }
    if (precision == SCESS_PRECISION_MIXED) c.tensor_cores().check_error();
  });
}

int scess_f12b_coupling(scess_ctx *ctx, const double *eri, const double *f12,
                        const double *f12_repulsion, const double *C, int64_t nmo, int64_t nocc,
                        int32_t precision, double *residual_out, double *energy_out) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(eri, "eri");
    need(f12, "f12");
    need(f12_repulsion, "f12_repulsion");
    need(C, "C");
    need(residual_out, "residual_out");
    need(energy_out, "energy_out");
    if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
      throw Error(SCESS_ERR_INVALID, "bad precision");
    const scess::Backend be =
        precision == SCESS_PRECISION_MIXED ? scess::Backend::TENSOR : scess::Backend::FP64;
    const int64_t N = nmo, o = nocc, v = N - o, N2 = N * N, N3 = N2 * N;
    // Host slices (Slice<> of CCSD_F12b.cpp:85-87): f12(k,l,r,s) and
    // f12_repulsion(k,l,a,b); the eri block (a,b,r,s) is a view of the uploaded eri.
    std::vector<double> f12_klrs((size_t)(o * o * N2)), rep_klab((size_t)(o * o * v * v));
    for (int64_t s_ = 0; s_ < N; s_++)
      for (int64_t r = 0; r < N; r++)
        for (int64_t l = 0; l < o; l++)
          for (int64_t k = 0; k < o; k++)
            f12_klrs[(size_t)(k + o * (l + o * (r + N * s_)))] = f12[k + N * l + N2 * r + N3 * s_];
    for (int64_t b = 0; b < v; b++)
      for (int64_t a = 0; a < v; a++)
        for (int64_t l = 0; l < o; l++)
          for (int64_t k = 0; k < o; k++)
            rep_klab[(size_t)(k + o * (l + o * (a + v * b)))] =
                f12_repulsion[k + N * l + N2 * (o + a) + N3 * (o + b)];
    host_finite(f12_klrs.data(), (int64_t)f12_klrs.size(), "f12");
    host_finite(rep_klab.data(), (int64_t)rep_klab.size(), "f12_repulsion");
    host_finite(C, o * o * v * v, "C");
    scess::DTensor d_eri = device_eri(c, eri, N);
    scess::DTensor dF({o, o, N, N}), V({o, o, v, v}), dC({o, o, v, v});
    scess::upload(c, dF.p(), f12_klrs.data(), o * o * N2);
    scess::upload(c, V.p(), rep_klab.data(), o * o * v * v);
    scess::upload(c, dC.p(), C, o * o * v * v);
    scess::TV eri_abrs;  // eri(o+a, o+b, r, s)
    eri_abrs.p = d_eri.p() + o + o * N;
    eri_abrs.nd = 4;
    const int64_t ee[4] = {v, v, N, N}, es[4] = {1, N, N2, N3};
    std::memcpy(eri_abrs.ext, ee, sizeof(ee));
    std::memcpy(eri_abrs.str, es, sizeof(es));
    // V_klab -= abrs,klrs->klab                                                 :85-87
    scess::einsum(c, "abrs,klrs->klab", -1.0, eri_abrs, dF.v, 1.0, V.v, be);
    // residual = F(C + V), energy = F(C), F(X) = 3/8 X + 1/8 X^(i<->j)    :31-35, :90-91
    scess::DTensor X({o, o, v, v}), E({o, o, v, v});
    scess::permute(c, "ijab->ijab", 1.0, V.v, 0.0, X.v);
    scess::permute(c, "ijab->ijab", 1.0, dC.v, 1.0, X.v);
    scess::permute(c, "ijab->ijab", 0.375, dC.v, 0.0, E.v);
    scess::permute(c, "jiab->ijab", 0.125, dC.v, 1.0, E.v);
    scess::permute(c, "ijab->ijab", 0.375, X.v, 0.0, V.v);
    scess::permute(c, "jiab->ijab", 0.125, X.v, 1.0, V.v);
    scess::download(c, residual_out, V.p(), o * o * v * v);
    scess::download(c, energy_out, E.p(), o * o * v * v);
    if (precision == SCESS_PRECISION_MIXED) c.tensor_cores().check_error();
  });
}

int scess_mp2_energy(scess_ctx *ctx, const double *mo_eri, const double *eps, int64_t nmo,
                     int64_t nocc, double *e_mp2) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(mo_eri, "mo_eri");
    need(eps, "eps");
    need(e_mp2, "e_mp2");
    host_finite(eps, nmo, "eps");
    const int64_t N = nmo, o = nocc, v = N - o, N2 = N * N;
    scess::DTensor g = device_eri(c, mo_eri, N);
    scess::DTensor de({N});
    scess::upload(c, de.p(), eps, N);
    // (ia|jb) = g(i, o+a, j, o+b)                                          RHF.cpp:334
    scess::mp2_energy(o, v, g.p() + o * N + o * N2 * N, 1, N, N2, N2 * N, de.p(), c.partials,
                      c.dscalars, c.stream);
    SCESS_CUDA(cudaMemcpyAsync(c.hscalars, c.dscalars, sizeof(double), cudaMemcpyDeviceToHost,
                               c.stream));
    c.sync();
    *e_mp2 = c.hscalars[0];
  });
}

int scess_mp2_energy_ao(scess_ctx *ctx, const double *ao_eri, const double *C, const double *eps,
                        int64_t nao, int64_t nmo, int64_t nocc, int32_t precision,
                        double *e_mp2) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(ao_eri, "ao_eri");
    need(C, "C");
    need(eps, "eps");
    need(e_mp2, "e_mp2");
    if (nao <= 0) throw Error(SCESS_ERR_INVALID, "bad dimensions");
    if (precision != SCESS_PRECISION_FP64 && precision != SCESS_PRECISION_MIXED)
      throw Error(SCESS_ERR_INVALID, "bad precision");
    host_finite(eps, nmo, "eps");
    const scess::Backend be =
        precision == SCESS_PRECISION_MIXED ? scess::Backend::TENSOR : scess::Backend::FP64;
    const int64_t n = nao, o = nocc, v = nmo - nocc;
    scess::DTensor dC({n, nmo});
    scess::upload(c, dC.p(), C, n * nmo);
    device_finite(c, dC.p(), n * nmo, "C");
    const scess::TV Cocc = scess::cm(dC.p(), {n, o}), Cvirt = scess::cm(dC.p() + n * o, {n, v});
    // (a i|b j) = TransformTEI(aoERI, C_virt, C_occ, C_virt, C_occ), the last
    // index first                                                            RHF.cpp:282-283
    scess::DTensor x({n, n, n, n});
    scess::upload(c, x.p(), ao_eri, n * n * n * n);
    device_finite(c, x.p(), n * n * n * n, "ao_eri");
    scess::DTensor y({n, n, n, o});
    scess::einsum(c, "mnkl,ls->mnks", 1.0, x.v, Cocc, 0.0, y.v, be);
    x = scess::DTensor({n, n, v, o});
    scess::einsum(c, "mnks,kr->mnrs", 1.0, y.v, Cvirt, 0.0, x.v, be);
    y = scess::DTensor({n, o, v, o});
    scess::einsum(c, "mnrs,nq->mqrs", 1.0, x.v, Cocc, 0.0, y.v, be);
    x = scess::DTensor({v, o, v, o});
    scess::einsum(c, "mqrs,mp->pqrs", 1.0, y.v, Cvirt, 0.0, x.v, be);
    scess::DTensor de({nmo});
    scess::upload(c, de.p(), eps, nmo);
    // (ia|jb) = aibj(a, i, b, j)                                            RHF.cpp:292
    scess::mp2_energy(o, v, x.p(), v, 1, v * o * v, v * o, de.p(), c.partials, c.dscalars,
                      c.stream);
    SCESS_CUDA(cudaMemcpyAsync(c.hscalars, c.dscalars, sizeof(double), cudaMemcpyDeviceToHost,
                               c.stream));
    c.sync();
    *e_mp2 = c.hscalars[0];
    if (precision == SCESS_PRECISION_MIXED) c.tensor_cores().check_error();
  });
}

int scess_ccsd_so_solve(scess_ctx *ctx, const double *mo_eri, const double *eps, int64_t nmo,
                        int64_t nocc, int32_t diis, int32_t triples, double *t1_out,
                        double *t2_out, double *g_out, scess_rccsd_result *result) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(mo_eri, "mo_eri");
    need(eps, "eps");
    need(t1_out, "t1_out");
    need(t2_out, "t2_out");
    need(result, "result");
    host_finite(eps, nmo, "eps");
    const int64_t N = 2 * nmo, o = 2 * nocc, v = N - o;
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    scess::DTensor g({N, N, N, N});
    {
      scess::DTensor chem = device_eri(c, mo_eri, nmo);
      scess::so_antisymmetrise(c, chem.p(), nmo, g.p());
    }
    scess::DTensor de({nmo}), t1({o, v}), t2({o, o, v, v});
    scess::upload(c, de.p(), eps, nmo);
    const scess::SoResult r =
        scess::so_ccsd(c, g.p(), de.p(), nmo, nocc, diis != 0, triples != 0, ctl, t1.p(), t2.p());
    scess::download(c, t1_out, t1.p(), o * v);
    scess::download(c, t2_out, t2.p(), o * o * v * v);
    if (g_out) scess::download(c, g_out, g.p(), N * N * N * N);
    *result = scess_rccsd_result{};
    result->E_CCSD = r.E_CCSD;
    result->E_T = r.E_T;
    result->converged = r.converged ? 1 : 0;
    result->iterations = r.iterations;
    result->last_dE = r.last_dE;
  });
}

int scess_ccsd_so_triples(scess_ctx *ctx, const double *g, const double *eps, int64_t nmo,
                          int64_t nocc, const double *t1, const double *t2, double *e_t) {
  return guard(ctx, [&](scess::Ctx &c) {
    check_shape(nmo, nocc);
    need(g, "g");
    need(eps, "eps");
    need(t1, "t1");
    need(t2, "t2");
    need(e_t, "e_t");
    host_finite(eps, nmo, "eps");
    const int64_t N = 2 * nmo, o = 2 * nocc, v = N - o;
    scess::Control ctl;
    ctl.cancel = c.cancel;
    ctl.user = c.user;
    scess::DTensor dg = device_eri(c, g, N);
    scess::DTensor de({nmo}), d1({o, v}), d2({o, o, v, v});
    scess::upload(c, de.p(), eps, nmo);
    scess::upload(c, d1.p(), t1, o * v);
    scess::upload(c, d2.p(), t2, o * o * v * v);
    device_finite(c, d1.p(), o * v, "t1");
    device_finite(c, d2.p(), o * o * v * v, "t2");
    *e_t = scess::so_triples(c, dg.p(), de.p(), nmo, nocc, d1.p(), d2.p(), ctl);
  });
}

}  // extern "C"
