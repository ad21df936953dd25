// Host-side engine: context, device memory, tensor views and the einsum compiler.
#pragma once
#include <chrono>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.h"

namespace scess {

// Owning device allocation (freed on destruction).
struct Ctx;

// Large device blocks released while an API call of their context runs are
// kept by that context (exact sizes) instead of going back through cudaFree,
// which synchronises the whole device; later allocations of the same size in
// the same context reuse them.  All of a context's kernels run on its one
// stream, so a reused block's earlier work precedes its new work.  The cache
// is emptied when an allocation fails and with the context.
class BlockCache {
 public:
  static constexpr size_t kMinBytes = size_t(1) << 20;
  static constexpr size_t kMaxCached = size_t(96) << 30;
  void *take(size_t bytes);
  bool give(void *p, size_t bytes);  // false: the caller frees it
  size_t flush();  // frees every cached block; returns the bytes freed
  size_t bytes() const { return total_; }

 private:
  std::multimap<size_t, void *> free_;
  size_t total_ = 0;
};

// Internal tuning switches, for tests and tuning runs only: the environment
// variable SCESS_TUNE holds "key=value" pairs separated by commas, read at
// every call.  Keys: t_nb (virtual block size of (T), both forms; default: the
// size chosen from o and v), t_kbd (K blocks of 64 per TMEM drain in the
// mixed (T) launch: 1, 2 or 4) and t_wbuf (W buffers of the mixed (T): 1 or 3).
// Returns `def` for an unset key.
int64_t tune_value(const char *key, int64_t def);
// TMEM drain cadence of the mixed (T) launch (K blocks of 64 per drain).
constexpr int kTriplesKbd = 4;
// W buffers of the mixed (T): 1 (the groups add into one with L2 reductions) or
// 3 (one per group, plain stores).
constexpr int kTriplesWBuffers = 1;

// The context whose API call runs on this thread (null outside calls).
Ctx *current_ctx();
struct CurrentCtx {
  Ctx *prev;
  explicit CurrentCtx(Ctx *c);
  ~CurrentCtx();
};

class DevMem {
 public:
  DevMem() = default;
  explicit DevMem(size_t bytes) { alloc(bytes); }
  ~DevMem() { release(); }
  DevMem(const DevMem &) = delete;
  DevMem &operator=(const DevMem &) = delete;
  DevMem(DevMem &&o) noexcept : p_(o.p_), bytes_(o.bytes_), owner_(o.owner_) {
    o.p_ = nullptr;
    o.bytes_ = 0;
    o.owner_ = nullptr;
  }
  DevMem &operator=(DevMem &&o) noexcept {
    if (this != &o) {
      release();
      p_ = o.p_;
      bytes_ = o.bytes_;
      owner_ = o.owner_;
      o.p_ = nullptr;
      o.bytes_ = 0;
      o.owner_ = nullptr;
    }
    return *this;
  }
  void alloc(size_t bytes);
  void release();
  template <class T> T *as() const { return static_cast<T *>(p_); }
  double *d() const { return static_cast<double *>(p_); }
  size_t bytes() const { return bytes_; }

 private:
  void *p_ = nullptr;
  size_t bytes_ = 0;
  Ctx *owner_ = nullptr;  // context whose API call allocated it
};

// Strided view of an FP64 tensor in device memory: element (i_0, ..., i_{nd-1})
// lives at p[sum_d i_d * str[d]].
struct TV {
  double *p = nullptr;
  int nd = 0;
  int64_t ext[6] = {1, 1, 1, 1, 1, 1};
  int64_t str[6] = {0, 0, 0, 0, 0, 0};
  int64_t size() const {
    int64_t n = 1;
    for (int d = 0; d < nd; d++) n *= ext[d];
    return n;
  }
};
// Column-major (first index fastest) dense view.
TV cm(double *p, std::initializer_list<int64_t> ext);
// A dense column-major tensor that owns its memory.
struct DTensor {
  DevMem mem;
  TV v;
  DTensor() = default;
  DTensor(std::initializer_list<int64_t> ext);
  double *p() const { return v.p; }
  int64_t size() const { return v.size(); }
};

// Geometry of an einsum (label groups and offset tables), shared by backends.
struct EinsumPlan {
  int64_t M = 1, N = 1, K = 1;
  std::vector<int64_t> rowA, kA, colB, kB, rowC, colC;  // host copies
  std::shared_ptr<DevMem> dev;  // rowA | kA | colB | kB | rowC | colC on the device
  const int64_t *d_rowA = nullptr, *d_kA = nullptr, *d_colB = nullptr, *d_kB = nullptr;
  const int64_t *d_rowC = nullptr, *d_colC = nullptr;
  bool aUnitM = false, bUnitN = false, aUnitK = false, bUnitK = false;
  bool cUnitM = false, cUnitN = false;  // C's unit-stride label leads the M / N group
  // the operand offset tables as plain strides (offset = index * stride), or -1
  int64_t aRowStride = -1, aKStride = -1, bColStride = -1, bKStride = -1;
  // packing hints: rows r = pre + P (f + E post), f along the operand's
  // smallest-stride row label; dense: the gather is a permutation of src[0, n)
  int64_t aRowP = 1, aRowE = 1, bColP = 1, bColE = 1;
  bool aDense = false, bDense = false;
  std::string key;
  std::string spec;
  // content hashes of (rowA, kA) and (colB, kB), computed on first use: two
  // plans that gather an operand through equal tables pack it identically
  mutable uint64_t hashA = 0, hashB = 0;
};
class TcEngine;  // tensor-core (mixed precision) backend, gemm_tc.cu

// Forward-op record for the hand-written adjoint: every einsum / permute (and
// the residual's tau and PlusTranspose steps) issued while Ctx::tape is set is
// appended with its operand views; adjoint.cu sweeps the list in reverse.
struct TapeOp {
  enum Kind { EINSUM = 0, PERMUTE = 1, TAU = 2, PLUS_T = 3 } kind = EINSUM;
  std::string spec;
  double alpha = 1.0, beta = 0.0;
  TV A, B, C;
  int64_t o = 0, v = 0;
};
struct Tape {
  std::vector<TapeOp> ops;
};

// Per-call control: cancellation and the time limit.
struct Control {
  scess_cancel_fn cancel = nullptr;
  void *user = nullptr;
  double time_limit_s = 0.0;
  std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
  void poll() const;
};

// Optional per-kernel timing: CUDA events recorded on the launching stream
// around each instrumented launch, aggregated per kernel name (launches,
// device milliseconds, algorithmic FLOPs and bytes).
class KernelTimer {
 public:
  struct Agg {
    int64_t launches = 0;
    double ms = 0.0, flops = 0.0, bytes = 0.0;
  };
  bool on = false;
  ~KernelTimer();
  void begin(const char *name, double flops, double bytes, cudaStream_t s);
  void end(cudaStream_t s);
  void collect();  // waits for the recorded events and folds them into agg
  // host-side phase (wall clock, ms), reported beside the kernels as "host:<name>"
  void host(const char *name, double ms);
  void reset();
  std::map<std::string, Agg> agg;

 private:
  struct Rec {
    std::string name;
    cudaEvent_t a, b;
    double flops, bytes;
  };
  cudaEvent_t get();
  std::vector<Rec> recs_;
  std::vector<size_t> open_;  // records whose end() is pending (scopes nest)
  std::vector<cudaEvent_t> pool_;
};

// RAII helper: times the launches issued in its scope when the timer is on.
struct TimedScope {
  KernelTimer &t;
  cudaStream_t s;
  bool active;
  TimedScope(KernelTimer &tm, const char *name, double flops, double bytes, cudaStream_t st)
      : t(tm), s(st), active(tm.on) {
    if (active) t.begin(name, flops, bytes, s);
  }
  ~TimedScope() {
    if (active) t.end(s);
  }
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  scess_cancel_fn cancel = nullptr;
  scess_log_fn log = nullptr;
  void *user = nullptr;

  // einsum plans (offset tables), keyed by spec + operand geometry
  std::map<std::string, std::unique_ptr<EinsumPlan>> plans;
  DevMem workspace;          // split-K partials
  DevMem scratch;            // partial sums of reductions + device scalars
  double *partials = nullptr;
  double *dscalars = nullptr;  // 64 device doubles
  double *hscalars = nullptr;  // 64 pinned host doubles
  std::unique_ptr<TcEngine> tc;
  KernelTimer timer;
  Tape *tape = nullptr;  // recording target while an adjoint forward pass runs
  BlockCache blocks;     // released large device blocks (see BlockCache)
  // Device memory held by this context's calls (live blocks and the block
  // cache) and its cap (0 = none): an allocation beyond the cap fails with
  // SCESS_ERR_OOM as if the device were full (scess_ctx_set_memory_limit).
  size_t mem_held = 0, mem_limit = 0;

  explicit Ctx(int dev);
  ~Ctx();
  void sync() const { SCESS_CUDA(cudaStreamSynchronize(stream)); }
  double *ensure_workspace(int64_t doubles);
  void logf(int level, const char *fmt, ...) const;
  TcEngine &tensor_cores();
};

// FP64: DFMA engine.  MIXED: tensor cores for contractions large enough to pay
// for packing, FP64 for the rest.  TENSOR: tensor cores for every contraction.
enum class Backend { FP64 = 0, MIXED = 1, TENSOR = 2 };

// C[labels] = alpha * A[labels] B[labels] + beta * C   (spec "kcld,ilcd->ki").
// Backend::MIXED routes large contractions to the tcgen05 engine and keeps
// small ones in FP64.  `constA`/`constB` mark operands whose contents do not
// change during the call so that their tensor-core packing can be reused.
void einsum(Ctx &ctx, const char *spec, double alpha, const TV &A, const TV &B, double beta,
            const TV &C, Backend be = Backend::FP64, bool constA = false, bool constB = false);
// Y[out labels] = alpha * X[in labels] + beta * Y   (spec "kcai->akic").
void permute(Ctx &ctx, const char *spec, double alpha, const TV &X, double beta, const TV &Y);

const EinsumPlan &plan_einsum(Ctx &ctx, const char *spec, const TV &A, const TV &B, const TV &C);

// Upload helpers (synchronous w.r.t. the host buffer).
void upload(Ctx &ctx, double *dst, const double *src, int64_t n);
void download(Ctx &ctx, double *dst, const double *src, int64_t n);

}  // namespace scess
