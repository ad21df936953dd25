// Tensor-core (tcgen05 / TMEM / TMA) backend of the mixed-precision form.
//
// Operands are FP64 in HBM.  A pack kernel gathers them through offset tables
// (fusing the einsum permutation) and splits every value x into BF16 hi + lo
// (hi = bf16(x), lo = bf16(x - hi)); a packed operand is a row-major
// [rows_pad][2*Kpad] BF16 array holding hi in columns [0, Kpad) and lo in
// [Kpad, 2 Kpad).  The GEMM kernel runs three K segments hi*hi + hi*lo + lo*hi
// into one FP32 TMEM accumulator (the lo*lo term is below FP32 resolution) and
// its epilogue scatters alpha*acc + beta*C into the FP64 (or FP32) output.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <map>
#include <memory>
#include <string>

#include "engine.h"

namespace scess {

struct Packed {
  DevMem mem;
  int64_t rows = 0, rows_pad = 0, K = 0, Kpad = 0;
  __nv_bfloat16 *p() const { return mem.as<__nv_bfloat16>(); }
};

// Output of a tensor-core GEMM: element (m, n) of the product goes to
// C[baseC + rowC[m] + colC[n]] (tables on the device).
struct TcOut {
  void *C = nullptr;
  int fp32 = 0;  // 0: C is double, 1: C is float
  const int64_t *rowC = nullptr, *colC = nullptr;
  int64_t baseC = 0;
  double alpha = 1.0, beta = 0.0;
};

class TcEngine {
 public:
  explicit TcEngine(Ctx &ctx);
  ~TcEngine();
  // Large enough to pay for packing and a tensor-core launch.
  static bool worth_it(const EinsumPlan &pl);
  // einsum through the plan's offset tables (see einsum()).
  void contract(const EinsumPlan &pl, double alpha, const double *A, const double *B, double beta,
                double *C, bool constA, bool constB);
  // Pack rows x K values src[rowOff[r] + kOff[k]] into `out` (rows padded to a
  // multiple of `row_align`, K to a multiple of 64).  unitK: the source is
  // contiguous along k (load-coalescing hint).
  void pack(const double *src, const int64_t *rowOff, int64_t rows, const int64_t *kOff,
            int64_t K, bool unitK, int64_t row_align, Packed &out);
  // D(m, n) = sum_k A(rowA0 + m, k) B(rowB0 + n, k) for m < M, n < N, written
  // through `out`.  nseg = 3 (split hi/lo) or 1 (hi only, BF16 accuracy).
  void gemm(const Packed &A, int64_t rowA0, int64_t M, const Packed &B, int64_t rowB0, int64_t N,
            const TcOut &out, int nseg = 3, int force_splits = 0);
  // Tile width used for an N-column product (multiple of 16, <= 256).
  static int tile_n(int64_t N);
  // TMA descriptor of a packed operand with boxes of box_rows x 64.
  static CUtensorMap map_of(const Packed &p, int box_rows);
  // gemm() with prebuilt descriptors (mb must use box_rows == tile_n(N)); no split-K.
  void gemm_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t rowA0,
                 int64_t M, int64_t rowB0, int64_t N, const TcOut &out, int nseg = 3,
                 cudaStream_t stream = nullptr);
  // Device error word set by bounded waits inside the kernels (0 = fine).
  void check_error();
  // Drops cached packings of constant operands (called at the end of every
  // top-level call: the cache is keyed by device pointer).
  void clear_cache() { cache_.clear(); }

 private:
  Ctx &ctx_;
  std::map<std::string, std::unique_ptr<Packed>> cache_;
  Packed tmpA_, tmpB_;
  DevMem partial_;
  DevMem err_;
};

// Raw launchers.
void tc_gemm_launch(const __nv_bfloat16 *A, int64_t a_rows_pad, const __nv_bfloat16 *B,
                    int64_t b_rows_pad, int64_t Kpad, int64_t rowA0, int64_t M, int64_t rowB0,
                    int64_t N, const TcOut &out, int nseg, int splits, float *partial,
                    unsigned *err, cudaStream_t stream);
void tc_gemm_launch_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t rowA0,
                         int64_t M, int64_t rowB0, int64_t N, int bn, const TcOut &out, int nseg,
                         int splits, float *partial, unsigned *err, cudaStream_t stream);

}  // namespace scess
