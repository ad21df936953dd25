// Tensor-core (tcgen05 / TMEM / TMA) backend of the mixed-precision form.
//
// Operands are FP64 in HBM.  A pack kernel gathers them through offset tables
// (fusing the einsum permutation) and splits every value into a 16-bit hi + lo
// pair; a packed operand is a row-major [rows_pad][2*Kpad] array holding hi in
// columns [0, Kpad) and lo in [Kpad, 2 Kpad).  Two operand formats:
//   FP16 (default): x is first scaled by a power of two s chosen on the device
//     from max|x| so that max|x| s lies in [2^14, 2^15); hi = fp16(x s),
//     lo = fp16(x s - hi).  11 significant bits each: |x s - hi - lo| <= 2^-22 |x s|.
//   BF16: hi = bf16(x), lo = bf16(x - hi), no scaling (|x - hi - lo| <= 2^-16 |x|).
// The GEMM kernel runs three K segments hi*hi + hi*lo + lo*hi into one FP32
// TMEM accumulator (lo*lo is dropped) and its epilogue scatters
// alpha/(sA sB) * acc + beta*C into the FP64 (or FP32) output.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <map>
#include <vector>
#include <memory>
#include <string>

#include "engine.h"

namespace scess {

enum class TcFormat { BF16 = 0, FP16 = 1 };

struct Packed {
  DevMem mem;
  DevMem aux;  // [0]: max|x| as float bits (uint32), [8]: scale s (double)
  int64_t rows = 0, rows_pad = 0, K = 0, Kpad = 0;
  TcFormat fmt = TcFormat::FP16;
  __nv_bfloat16 *p() const { return mem.as<__nv_bfloat16>(); }
  const double *scale() const { return aux.bytes() ? reinterpret_cast<const double *>(aux.as<char>() + 8) : nullptr; }
};

// Output of a tensor-core GEMM: element (m, n) of the product goes to
// C[baseC + rowC[m] + colC[n]] (tables on the device).
struct TcOut {
  void *C = nullptr;
  int fp32 = 0;  // 0: C is double, 1: C is float
  const int64_t *rowC = nullptr, *colC = nullptr;
  int64_t baseC = 0;
  double alpha = 1.0, beta = 0.0;
  // Scales of the packed operands (device doubles, null = 1): the product is
  // divided by scaleA * scaleB.
  const double *scaleA = nullptr, *scaleB = nullptr;
};

// A launch of several same-shaped GEMMs ("problems" (y, z, g) in
// [0,ny) x [0,nz) x [0,ng), ng <= 3), each summing up to four K segments whose
// operands are rows of packed tensors: segment s of problem (y, z, g)
// multiplies rows rowA0[g] + y rowAy[g] + z rowAz[g] (+ m) of maps[mapA] with
// rows rowB0[g] + y rowBy[g] + z rowBz[g] (+ n) of maps[mapB] over Kpad
// columns, negated when `negate`.  Problem (y, z, g) writes at offset
// y cy[g] + z cz[g] + cg[g] (plus the tables).  All segments' operand pairs
// must carry the same scale product (the epilogue unscales once).
struct TcSegment {
  int mapA = 0, mapB = 1;
  int64_t Kpad = 0;
  // K block of this segment: 0 = the kernel's; 32 in the 64-wide kernel (its
  // maps then have 32-wide boxes and Kpad is a multiple of 32)
  int bk = 0;
  bool negate = false;
  int64_t rowA0[3] = {0, 0, 0}, rowAy[3] = {0, 0, 0}, rowAz[3] = {0, 0, 0};
  int64_t rowB0[3] = {0, 0, 0}, rowBy[3] = {0, 0, 0}, rowBz[3] = {0, 0, 0};
};
struct TcProblemSet {
  CUtensorMap maps[6];
  int nmaps = 0;
  int64_t M = 0, N = 0;
  int ny = 1, nz = 1, ng = 1;
  int nseg = 1;
  TcSegment seg[4];
  int64_t cy[3] = {0, 0, 0}, cz[3] = {0, 0, 0};
  int64_t cg[3] = {0, 0, 0};
  // K blocks per TMEM drain: 1, 2 or 4 (fewer drains, more products
  // accumulated in TMEM between drains).  A K block is k_block(bn) wide.
  int kbd = 1;
  // group g computes only its problems with y >= z (requires ny == nz)
  bool tri[3] = {false, false, false};
  // tile width: 128, or 256 (B-side maps must then have 256-row boxes; half the
  // shared-memory traffic per FLOP for the A operand).  All maps must have
  // k_block(bn)-wide boxes: map_of(p, rows, k_block(bn)), and bk must say so.
  int bn = 128;
  int bk = 64;
  // bn = 256, bk = 64 only: run each 256 x 256 unit on a cluster pair of SMs
  // (tcgen05 cta_group::2, M = 256); the B-side maps then have 128-row boxes
  // (each CTA stages half of the unit's B columns) and so do the A-side maps
  bool pair = false;
  // per-group output tables (null: the TcOut tables)
  const int64_t *rowC[3] = {nullptr, nullptr, nullptr};
  const int64_t *colC[3] = {nullptr, nullptr, nullptr};
  // group g writes along columns (lanes over columns, through shared memory):
  // for FP32 outputs with beta = 0 whose unit-stride index is a column index
  // (with store_quads also for beta = 1, as L2 reductions)
  bool store_by_column[3] = {false, false, false};
  // ... and every aligned quad of columns (4 c .. 4 c + 3) goes to 4 contiguous
  // floats at a 16-byte aligned address (vector stores)
  bool store_quads[3] = {false, false, false};
  // launch as a programmatic dependent of the stream's previous kernel (which
  // must call griddepcontrol.launch_dependents): the prologue and the MMAs run
  // while that kernel finishes, the epilogue waits for it before its first
  // store.  Only for a launch whose operands and tables that kernel does not
  // write (the (T) launches after the first, behind an energy kernel).
  bool pdl = false;
};

// Bounds of the kernels' pipeline waits.  The defaults are the production
// ones; the diagnostics entry point arms a short bound and a withheld first
// stage for one launch, to exercise the expiry path.
struct TcWaitDiag {
  long long wait_cycles = 1ll << 32;
  bool withhold_first = false;
};

class TcEngine {
 public:
  explicit TcEngine(Ctx &ctx);
  ~TcEngine();
  // Large enough to pay for packing and a tensor-core launch.
  static bool worth_it(const EinsumPlan &pl);
  // The FP64 engine's table GEMM (TableGemm: C[baseC + rowC[m] + colC[n]] =
  // alpha sum_k A[baseA + rowA[m] + kA[k]] B[baseB + colB[n] + kB[k]] + beta C)
  // on the tensor cores: both operands packed through their tables, split
  // hi/lo, FP32 accumulation; `name` labels the kernel timer.
  void table_gemm(const TableGemm &g, const char *name);
  // einsum through the plan's offset tables (see einsum()).
  void contract(const EinsumPlan &pl, double alpha, const double *A, const double *B, double beta,
                double *C, bool constA, bool constB);
  // Pack rows x K values src[rowOff[r] + kOff[k]] into `out` (rows padded to a
  // multiple of `row_align`, K to a multiple of 64).  unitK: the source is
  // contiguous along k (load-coalescing hint).  rs, ks >= 0: the tables are
  // rowOff[r] = r rs, kOff[k] = k ks (they are then not read).  rP, rE: tiles
  // take 32 rows r = pre + rP (f + rE post) along one label of the row group
  // (rE = 0: consecutive rows).  dense: the gather visits src[0, rows K) once.
  void pack(const double *src, const int64_t *rowOff, int64_t rows, const int64_t *kOff,
            int64_t K, bool unitK, int64_t row_align, Packed &out, int64_t rs = -1,
            int64_t ks = -1, int64_t rP = 1, int64_t rE = 0, bool dense = false);
  // max|x| over the same gather, folded into *maxbits (float bits, atomic max:
  // several calls into one word give the max over all their tensors).
  void maxabs_into(const double *src, const int64_t *rowOff, int64_t rows, const int64_t *kOff,
                   int64_t K, bool unitK, unsigned *maxbits);
  // pack() with the FP16 scale taken from a given max word (so that several
  // packs share one scale), optionally negating the values (exact).
  // K is padded to a multiple of k_align (64, or 32 for segments with 32-wide
  // K blocks).
  void pack_with_max(const double *src, const int64_t *rowOff, int64_t rows, const int64_t *kOff,
                     int64_t K, bool unitK, int64_t row_align, const unsigned *maxbits,
                     bool negate, Packed &out, int64_t k_align = 64);
  TcFormat format() const { return fmt_; }
  // D(m, n) = sum_k A(rowA0 + m, k) B(rowB0 + n, k) for m < M, n < N, written
  // through `out`.  nseg = 3 (split hi/lo) or 1 (hi only, BF16 accuracy).
  void gemm(const Packed &A, int64_t rowA0, int64_t M, const Packed &B, int64_t rowB0, int64_t N,
            const TcOut &out, int nseg = 3, int force_splits = 0);
  // Tile width used for an N-column product (multiple of 16, <= 256).
  static int tile_n(int64_t N);
  // TMA descriptor of a packed operand with boxes of box_rows x bk (bk = 64:
  // SWIZZLE_128B, bk = 32: SWIZZLE_64B).
  static CUtensorMap map_of(const Packed &p, int box_rows, int bk = 64);
  // K block (16-bit values per stage row) of the kernel with tile width bn.
  static int k_block(int bn);
  // whether this device runs the cluster-pair form of the 256 x 64 kernel
  // (TcProblemSet::pair)
  static bool pair_available();
  // TcOut scale pointers of a product of two packed operands.
  static void set_scales(TcOut &out, const Packed &A, const Packed &B) {
    out.scaleA = A.scale();
    out.scaleB = B.scale();
  }
  // gemm() with prebuilt descriptors (mb must use box_rows == tile_n(N)); no split-K.
  // Grouped launch (see TcProblemSet); flops: algorithmic FLOPs for the timer.
  void gemm_grouped(const TcProblemSet &ps, const TcOut &out, double flops, const char *name,
                    cudaStream_t stream = nullptr);
  // Kreal: the unpadded K (algorithmic FLOPs for the kernel timer).
  void gemm_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t Kreal,
                 int64_t rowA0, int64_t M, int64_t rowB0, int64_t N, const TcOut &out,
                 int nseg = 3, cudaStream_t stream = nullptr);
  // Device error word set by bounded waits inside the kernels (0 = fine).
  void check_error();
  // The next launch bounds its waits by wait_cycles and withholds its first
  // operand stage (its MMA thread's wait then runs out).
  void arm_wait_expiry(long long wait_cycles) {
    diag_.wait_cycles = wait_cycles;
    diag_.withhold_first = true;
  }
  // Cached packings of constant operands are keyed by device pointer and
  // tagged with the owner that keeps those pointers alive: a resident
  // RccsdState (its address) or 0 for a single C-ABI call.  clear_cache(owner)
  // drops the owner's entries; owner changes with set_cache_owner().
  void set_cache_owner(const void *owner) { owner_ = owner; }
  void clear_cache(const void *owner);

  // max|x| of a whole tensor, reduced once and shared by every pack whose
  // gather starts at that tensor's base pointer (each reads a subset of it,
  // so the shared maximum bounds its own; the FP16 scale is a power of two
  // that keeps every packed value in range).  For operands a call packs
  // several times in different orders (t2 and tau in a residual): one flat
  // pass instead of one gathered pass per pack, and one pack for every
  // einsum that gathers the tensor through equal tables.  The caller keeps
  // the tensor unchanged until clear_max_hints().
  void add_max_hint(const double *p, int64_t n);
  void clear_max_hints();

 private:
  Ctx &ctx_;
  TcFormat fmt_ = TcFormat::FP16;
  std::map<std::string, std::pair<const void *, std::unique_ptr<Packed>>> cache_;
  const void *owner_ = nullptr;
  const char *timer_name_ = nullptr;
  Packed tmpA_, tmpB_;
  struct MaxHint {
    const double *p;
    int slot;
  };
  std::vector<MaxHint> hints_;
  // packs of hinted tensors, by source and gather: a second einsum that
  // gathers the same tensor through equal tables reuses the first one's pack
  // (dropped with the hints)
  std::map<std::string, std::unique_ptr<Packed>> reuse_;
  DevMem hint_words_;  // one max word per hint slot
  DevMem partial_;
  DevMem err_;
  TcWaitDiag diag_;
  TcWaitDiag take_diag();
};

// Raw launchers.
void tc_gemm_launch_grouped(const TcProblemSet &ps, TcFormat fmt, const TcOut &out, int nseg,
                            int splits, float *partial, unsigned *err, cudaStream_t stream,
                            const TcWaitDiag &diag = TcWaitDiag());
void tc_gemm_launch_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t rowA0,
                         int64_t M, int64_t rowB0, int64_t N, int bn, TcFormat fmt,
                         const TcOut &out, int nseg, int splits, float *partial, unsigned *err,
                         cudaStream_t stream, const TcWaitDiag &diag = TcWaitDiag());

}  // namespace scess
