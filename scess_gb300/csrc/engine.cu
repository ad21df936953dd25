// Host engine: device memory, context, einsum compiler (spec -> offset-table GEMM).
#include <algorithm>
#include <cstdarg>
#include <cstdlib>
#include <cstring>

#include "engine.h"
#include "gemm_tc.h"

namespace scess {

std::atomic<long long> g_launches{0};

namespace {
thread_local Ctx *t_ctx = nullptr;
}

Ctx *current_ctx() { return t_ctx; }

int64_t tune_value(const char *key, int64_t def) {
  const char *env = std::getenv("SCESS_TUNE");
  if (!env) return def;
  const size_t kl = std::strlen(key);
  for (const char *p = env; *p;) {
    const char *end = std::strchr(p, ',');
    if (!end) end = p + std::strlen(p);
    if ((size_t)(end - p) > kl && std::strncmp(p, key, kl) == 0 && p[kl] == '=')
      return std::strtoll(p + kl + 1, nullptr, 10);
    p = *end ? end + 1 : end;
  }
  return def;
}
CurrentCtx::CurrentCtx(Ctx *c) : prev(t_ctx) { t_ctx = c; }
CurrentCtx::~CurrentCtx() { t_ctx = prev; }

void *BlockCache::take(size_t bytes) {
  auto it = free_.find(bytes);
  if (it == free_.end()) return nullptr;
  void *p = it->second;
  free_.erase(it);
  total_ -= bytes;
  return p;
}

bool BlockCache::give(void *p, size_t bytes) {
  if (bytes < kMinBytes || total_ + bytes > kMaxCached) return false;
  free_.emplace(bytes, p);
  total_ += bytes;
  return true;
}

size_t BlockCache::flush() {
  for (auto &kv : free_) cudaFree(kv.second);
  free_.clear();
  const size_t t = total_;
  total_ = 0;
  return t;
}

namespace {
// Frees the context's cached blocks (after its queued work) and stops counting them.
void flush_cache(Ctx *c) {
  cudaStreamSynchronize(c->stream);
  const size_t freed = c->blocks.flush();
  c->mem_held -= std::min(freed, c->mem_held);
}
}  // namespace

void DevMem::alloc(size_t bytes) {
  release();
  if (bytes == 0) return;
  Ctx *c = current_ctx();
  if (c && bytes >= BlockCache::kMinBytes) {
    if (void *p = c->blocks.take(bytes)) {  // (cached bytes are already counted as held)
      p_ = p;
      bytes_ = bytes;
      owner_ = c;
      return;
    }
  }
  if (c && c->mem_limit) {
    if (c->mem_held + bytes > c->mem_limit && c->blocks.bytes() > 0) flush_cache(c);
    if (c->mem_held + bytes > c->mem_limit)
      throw Error(SCESS_ERR_OOM, "device memory limit of the context reached: " +
                                     std::to_string(c->mem_held) + " B held + " +
                                     std::to_string(bytes) + " B requested > " +
                                     std::to_string(c->mem_limit) + " B");
  }
  cudaError_t e = cudaMalloc(&p_, bytes);
  if (e == cudaErrorMemoryAllocation && c && c->blocks.bytes() > 0) {
    cudaGetLastError();
    flush_cache(c);
    e = cudaMalloc(&p_, bytes);
  }
  if (e != cudaSuccess) {
    p_ = nullptr;
    cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? SCESS_ERR_OOM : SCESS_ERR_CUDA,
                "cudaMalloc(" + std::to_string(bytes) + " B): " + cudaGetErrorString(e));
  }
  bytes_ = bytes;
  owner_ = c;
  if (c) c->mem_held += bytes;
}

void DevMem::release() {
  if (p_) {
    Ctx *c = current_ctx();
    if (c && owner_ == c) {
      if (!c->blocks.give(p_, bytes_)) {
        cudaFree(p_);
        c->mem_held -= std::min(bytes_, c->mem_held);
      }
    } else {
      cudaFree(p_);
    }
  }
  p_ = nullptr;
  bytes_ = 0;
  owner_ = nullptr;
}

TV cm(double *p, std::initializer_list<int64_t> ext) {
  TV t;
  t.p = p;
  t.nd = (int)ext.size();
  int64_t s = 1;
  int d = 0;
  for (int64_t e : ext) {
    t.ext[d] = e;
    t.str[d] = s;
    s *= e;
    d++;
  }
  return t;
}

DTensor::DTensor(std::initializer_list<int64_t> ext) {
  int64_t n = 1;
  for (int64_t e : ext) n *= e;
  mem.alloc((size_t)std::max<int64_t>(n, 1) * sizeof(double));
  v = cm(mem.d(), ext);
}

void Control::poll() const {
  if (cancel && cancel(user)) throw Error(SCESS_ERR_CANCELLED, "cancelled by the caller");
  if (time_limit_s > 0.0) {
    const double el =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    if (el > time_limit_s) throw Error(SCESS_ERR_TIMEOUT, "time limit exceeded");
  }
}

Ctx::Ctx(int dev) : device(dev) {
  int n = 0;
  SCESS_CUDA(cudaGetDeviceCount(&n));
  if (dev < 0 || dev >= n) throw Error(SCESS_ERR_INVALID, "no CUDA device " + std::to_string(dev));
  cudaDeviceProp prop;
  SCESS_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    throw Error(SCESS_ERR_UNSUPPORTED, std::string("device is ") + prop.name + " (sm_" +
                                           std::to_string(prop.major) + std::to_string(prop.minor) +
                                           "); this library is built for sm_103a (GB300)");
  SCESS_CUDA(cudaSetDevice(dev));
  SCESS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  scratch.alloc((kDotBlocks + 64) * sizeof(double));
  partials = scratch.d();
  dscalars = partials + kDotBlocks;
  SCESS_CUDA(cudaMallocHost(&hscalars, 64 * sizeof(double)));
}

Ctx::~Ctx() {
  if (stream) cudaStreamSynchronize(stream);
  blocks.flush();
  tc.reset();
  plans.clear();
  workspace.release();
  scratch.release();
  if (hscalars) cudaFreeHost(hscalars);
  if (stream) cudaStreamDestroy(stream);
}

double *Ctx::ensure_workspace(int64_t doubles) {
  if (doubles <= 0) return workspace.d();
  if ((size_t)doubles * sizeof(double) > workspace.bytes()) {
    sync();
    workspace.alloc((size_t)doubles * sizeof(double));
  }
  return workspace.d();
}

void Ctx::logf(int level, const char *fmt, ...) const {
  if (!log) return;
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  log(level, buf, user);
}

TcEngine &Ctx::tensor_cores() {
  if (!tc) tc = std::make_unique<TcEngine>(*this);
  return *tc;
}

void upload(Ctx &ctx, double *dst, const double *src, int64_t n) {
  if (n <= 0) return;
  SCESS_CUDA(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                             ctx.stream));
  ctx.sync();
}

void download(Ctx &ctx, double *dst, const double *src, int64_t n) {
  if (n <= 0) return;
  SCESS_CUDA(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                             ctx.stream));
  ctx.sync();
}

KernelTimer::~KernelTimer() {
  for (auto &r : recs_) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : pool_) cudaEventDestroy(e);
}

cudaEvent_t KernelTimer::get() {
  if (!pool_.empty()) {
    cudaEvent_t e = pool_.back();
    pool_.pop_back();
    return e;
  }
  cudaEvent_t e;
  SCESS_CUDA(cudaEventCreate(&e));
  return e;
}

void KernelTimer::begin(const char *name, double flops, double bytes, cudaStream_t s) {
  Rec r{name, get(), get(), flops, bytes};
  SCESS_CUDA(cudaEventRecord(r.a, s));
  open_.push_back(recs_.size());
  recs_.push_back(r);
}

void KernelTimer::end(cudaStream_t s) {
  SCESS_CUDA(cudaEventRecord(recs_[open_.back()].b, s));
  open_.pop_back();
  if (open_.empty() && recs_.size() >= 4096) collect();
}

void KernelTimer::host(const char *name, double ms) {
  if (!on) return;
  Agg &a = agg[std::string("host:") + name];
  a.launches++;
  a.ms += ms;
}

void KernelTimer::collect() {
  for (auto &r : recs_) {
    SCESS_CUDA(cudaEventSynchronize(r.b));
    float ms = 0.0f;
    SCESS_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    Agg &g = agg[r.name];
    g.launches++;
    g.ms += ms;
    g.flops += r.flops;
    g.bytes += r.bytes;
    pool_.push_back(r.a);
    pool_.push_back(r.b);
  }
  recs_.clear();
}

void KernelTimer::reset() {
  collect();
  agg.clear();
}

// ---------------------------------------------------------------------------------------------
namespace {

struct Spec {
  std::string a, b, c;
};

Spec parse_spec(const char *spec, bool binary) {
  std::string s(spec);
  const size_t arrow = s.find("->");
  if (arrow == std::string::npos) throw Error(SCESS_ERR_INVALID, std::string("bad spec ") + spec);
  Spec r;
  std::string lhs = s.substr(0, arrow);
  r.c = s.substr(arrow + 2);
  if (binary) {
    const size_t comma = lhs.find(',');
    if (comma == std::string::npos) throw Error(SCESS_ERR_INVALID, std::string("bad spec ") + spec);
    r.a = lhs.substr(0, comma);
    r.b = lhs.substr(comma + 1);
  } else {
    r.a = lhs;
  }
  return r;
}

void geom_key(std::string &k, const TV &t) {
  k += '|';
  for (int d = 0; d < t.nd; d++) {
    k += std::to_string(t.ext[d]);
    k += ':';
    k += std::to_string(t.str[d]);
    k += ',';
  }
}

struct Lbl {
  char c;
  int64_t ext;
  int64_t sa, sb, sc;
};

// Stride s if the group's offsets are e * s for e = 0, 1, ... (labels of
// extent 1 ignored; 0 for an empty group), else -1.
int64_t affine_stride(const std::vector<Lbl> &ls, int which) {
  int64_t s = -1, next = -1;
  for (auto &l : ls) {
    if (l.ext == 1) continue;
    const int64_t st = which == 0 ? l.sa : (which == 1 ? l.sb : l.sc);
    if (s < 0) s = st;
    else if (st != next) return -1;
    next = st * l.ext;
  }
  return s < 0 ? 0 : s;
}

// Tiling hint for a gathered group: the label with the smallest stride in the
// operand (extent > 1).  Rows r = pre + P (f + E post) with f its index, P the
// product of the extents before it (group order) and E its extent.
void fast_label(const std::vector<Lbl> &ls, int which, int64_t &P, int64_t &E) {
  int64_t best = -1, bs = 0, prod = 1;
  P = 1;
  E = 1;
  for (auto &l : ls) {
    const int64_t st = which == 0 ? l.sa : l.sb;
    if (l.ext > 1 && (best < 0 || st < bs)) {
      best = 1;
      bs = st;
      P = prod;
      E = l.ext;
    }
    prod *= l.ext;
  }
  if (best < 0) E = prod;  // all extents 1
}

// Whether the labels of two groups together enumerate src[0, n) exactly once.
bool dense_gather(const std::vector<Lbl> &g1, const std::vector<Lbl> &g2, int which) {
  std::vector<std::pair<int64_t, int64_t>> d;  // (stride, extent)
  for (auto *g : {&g1, &g2})
    for (auto &l : *g)
      if (l.ext > 1) d.push_back({which == 0 ? l.sa : l.sb, l.ext});
  std::sort(d.begin(), d.end());
  int64_t next = 1;
  for (auto &x : d) {
    if (x.first != next) return false;
    next = x.first * x.second;
  }
  return true;
}

std::vector<int64_t> offsets(const std::vector<Lbl> &ls, int which) {
  int64_t n = 1;
  for (auto &l : ls) n *= l.ext;
  std::vector<int64_t> out((size_t)n);
  for (int64_t e = 0; e < n; e++) {
    int64_t r = e, off = 0;
    for (auto &l : ls) {
      const int64_t i = r % l.ext;
      r /= l.ext;
      off += i * (which == 0 ? l.sa : which == 1 ? l.sb : l.sc);
    }
    out[(size_t)e] = off;
  }
  return out;
}

}  // namespace

const EinsumPlan &plan_einsum(Ctx &ctx, const char *spec, const TV &A, const TV &B, const TV &C) {
  std::string key(spec);
  geom_key(key, A);
  geom_key(key, B);
  geom_key(key, C);
  auto it = ctx.plans.find(key);
  if (it != ctx.plans.end()) return *it->second;

  const Spec s = parse_spec(spec, true);
  if ((int)s.a.size() != A.nd || (int)s.b.size() != B.nd || (int)s.c.size() != C.nd)
    throw Error(SCESS_ERR_INVALID, std::string("rank mismatch in ") + spec);
  auto find = [](const std::string &l, char c) { return (int)l.find(c); };
  std::vector<Lbl> M, N, K;
  auto ext_of = [&](char c) -> int64_t {
    int64_t e = -1;
    int p;
    if ((p = find(s.a, c)) >= 0) e = A.ext[p];
    if ((p = find(s.b, c)) >= 0) {
      if (e >= 0 && e != B.ext[p]) throw Error(SCESS_ERR_INVALID, std::string("extent mismatch in ") + spec);
      e = B.ext[p];
    }
    if ((p = find(s.c, c)) >= 0) {
      if (e >= 0 && e != C.ext[p]) throw Error(SCESS_ERR_INVALID, std::string("extent mismatch in ") + spec);
      e = C.ext[p];
    }
    return e;
  };
  for (char c : s.c) {
    const int pa = find(s.a, c), pb = find(s.b, c), pc = find(s.c, c);
    if ((pa >= 0) == (pb >= 0))
      throw Error(SCESS_ERR_INVALID, std::string("unsupported batch/free label in ") + spec);
    Lbl l{c, ext_of(c), pa >= 0 ? A.str[pa] : 0, pb >= 0 ? B.str[pb] : 0, C.str[pc]};
    (pa >= 0 ? M : N).push_back(l);
  }
  for (char c : s.a) {
    if (find(s.c, c) >= 0) continue;
    const int pa = find(s.a, c), pb = find(s.b, c);
    if (pb < 0) throw Error(SCESS_ERR_INVALID, std::string("label only in A: ") + spec);
    K.push_back(Lbl{c, ext_of(c), A.str[pa], B.str[pb], 0});
  }
  for (char c : s.b)
    if (find(s.c, c) < 0 && find(s.a, c) < 0)
      throw Error(SCESS_ERR_INVALID, std::string("label only in B: ") + spec);

  auto pl = std::make_unique<EinsumPlan>();
  pl->key = key;
  pl->spec = spec;
  pl->rowA = offsets(M, 0);
  pl->rowC = offsets(M, 2);
  pl->colB = offsets(N, 1);
  pl->colC = offsets(N, 2);
  pl->kA = offsets(K, 0);
  pl->kB = offsets(K, 1);
  pl->M = (int64_t)pl->rowA.size();
  pl->N = (int64_t)pl->colB.size();
  pl->K = (int64_t)pl->kA.size();
  pl->aUnitM = !M.empty() && M[0].sa == 1;
  pl->bUnitN = !N.empty() && N[0].sb == 1;
  pl->aUnitK = !K.empty() && K[0].sa == 1;
  pl->cUnitM = !M.empty() && M[0].sc == 1;
  pl->cUnitN = !N.empty() && N[0].sc == 1;
  pl->bUnitK = false;
  for (auto &l : K)
    if (l.sb == 1) pl->bUnitK = true;
  fast_label(M, 0, pl->aRowP, pl->aRowE);
  fast_label(N, 1, pl->bColP, pl->bColE);
  pl->aDense = dense_gather(M, K, 0);
  pl->bDense = dense_gather(N, K, 1);
  pl->aRowStride = affine_stride(M, 0);
  pl->aKStride = affine_stride(K, 0);
  pl->bColStride = affine_stride(N, 1);
  pl->bKStride = affine_stride(K, 1);
  const size_t tot = pl->rowA.size() + pl->kA.size() + pl->colB.size() + pl->kB.size() +
                     pl->rowC.size() + pl->colC.size();
  pl->dev = std::make_shared<DevMem>(tot * sizeof(int64_t));
  int64_t *base = pl->dev->as<int64_t>();
  size_t off = 0;
  auto put = [&](const std::vector<int64_t> &v, const int64_t *&dptr) {
    dptr = base + off;
    if (!v.empty())
      // on the context's stream: the block may be a reused one that earlier
      // kernels on that stream still read (the host vectors live in the plan)
      SCESS_CUDA(cudaMemcpyAsync(base + off, v.data(), v.size() * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, ctx.stream));
    off += v.size();
  };
  put(pl->rowA, pl->d_rowA);
  put(pl->kA, pl->d_kA);
  put(pl->colB, pl->d_colB);
  put(pl->kB, pl->d_kB);
  put(pl->rowC, pl->d_rowC);
  put(pl->colC, pl->d_colC);
  auto &ref = *pl;
  ctx.plans.emplace(key, std::move(pl));
  return ref;
}

void einsum(Ctx &ctx, const char *spec, double alpha, const TV &A, const TV &B, double beta,
            const TV &C, Backend be, bool constA, bool constB) {
  if (ctx.tape) {
    TapeOp op;
    op.kind = TapeOp::EINSUM;
    op.spec = spec;
    op.alpha = alpha;
    op.beta = beta;
    op.A = A;
    op.B = B;
    op.C = C;
    ctx.tape->ops.push_back(op);
  }
  const EinsumPlan &pl = plan_einsum(ctx, spec, A, B, C);
  // short K and one short free side: an HBM-bound contraction, on the CUDA
  // cores in FP32 rather than packed for the tensor cores
  if (be != Backend::FP64 && pl.K <= kSkinnyMaxK && std::min(pl.M, pl.N) <= kSkinnyMaxS &&
      std::max(pl.M, pl.N) >= 4096 && !ctx.tape) {
    const bool small_is_a = pl.M <= pl.N;
    TableGemm g;
    g.A = A.p;
    g.B = B.p;
    g.C = C.p;
    g.rowA = pl.d_rowA;
    g.kA = pl.d_kA;
    g.colB = pl.d_colB;
    g.kB = pl.d_kB;
    g.rowC = pl.d_rowC;
    g.colC = pl.d_colC;
    g.M = pl.M;
    g.N = pl.N;
    g.K = pl.K;
    g.alpha = alpha;
    g.beta = beta;
    const std::string tname = std::string("skinny[") + spec + "]";
    TimedScope ts(ctx.timer, tname.c_str(), 2.0 * pl.M * pl.N * pl.K, 0.0, ctx.stream);
    skinny_table(g, small_is_a, small_is_a ? pl.cUnitM : pl.cUnitN, ctx.stream);
    return;
  }
  if ((be == Backend::MIXED && TcEngine::worth_it(pl)) || be == Backend::TENSOR) {
    ctx.tensor_cores().contract(pl, alpha, A.p, B.p, beta, C.p, constA, constB);
    return;
  }
  TableGemm g;
  g.A = A.p;
  g.B = B.p;
  g.C = C.p;
  g.rowA = pl.d_rowA;
  g.kA = pl.d_kA;
  g.colB = pl.d_colB;
  g.kB = pl.d_kB;
  g.rowC = pl.d_rowC;
  g.colC = pl.d_colC;
  g.M = pl.M;
  g.N = pl.N;
  g.K = pl.K;
  g.alpha = alpha;
  g.beta = beta;
  g.aUnitM = pl.aUnitM;
  g.bUnitN = pl.bUnitN;
  TimedScope ts(ctx.timer, (pl.N == 1 || pl.M == 1) ? "dgemv_table" : "dgemm_table",
                2.0 * pl.M * pl.N * pl.K, 0.0, ctx.stream);
  if (pl.N == 1 && pl.K > 0) {
    dgemv_table(g, ctx.stream);
    return;
  }
  if (pl.M == 1 && pl.K > 0) {  // C^T = B^T A^T
    TableGemm h = g;
    h.A = B.p;
    h.B = A.p;
    h.rowA = pl.d_colB;
    h.kA = pl.d_kB;
    h.colB = pl.d_rowA;
    h.kB = pl.d_kA;
    h.rowC = pl.d_colC;
    h.colC = pl.d_rowC;
    h.M = pl.N;
    h.N = 1;
    dgemv_table(h, ctx.stream);
    return;
  }
  double *ws = ctx.ensure_workspace(dgemm_table_workspace(g));
  dgemm_table(g, ws, ctx.stream);
}

void permute(Ctx &ctx, const char *spec, double alpha, const TV &X, double beta, const TV &Y) {
  if (ctx.tape) {
    TapeOp op;
    op.kind = TapeOp::PERMUTE;
    op.spec = spec;
    op.alpha = alpha;
    op.beta = beta;
    op.A = X;
    op.C = Y;
    ctx.tape->ops.push_back(op);
  }
  const Spec s = parse_spec(spec, false);
  if ((int)s.a.size() != X.nd || (int)s.c.size() != Y.nd)
    throw Error(SCESS_ERR_INVALID, std::string("rank mismatch in ") + spec);
  PermDesc d;
  d.nd = Y.nd;
  for (int k = 0; k < Y.nd; k++) {
    const int p = (int)s.a.find(s.c[k]);
    if (p < 0 || X.ext[p] != Y.ext[k]) throw Error(SCESS_ERR_INVALID, std::string("bad permute ") + spec);
    d.ext[k] = Y.ext[k];
    d.ys[k] = Y.str[k];
    d.xs[k] = X.str[p];
  }
  permute_add(d, alpha, X.p, beta, Y.p, ctx.stream);
}

}  // namespace scess
