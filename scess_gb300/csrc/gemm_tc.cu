// tcgen05 / TMEM / TMA tensor-core GEMM for sm_103a (split BF16 hi+lo, FP32 accumulate).
//
// One CTA computes a 128 x bn tile (bn <= 256, multiple of 16):
//   warp 0      TMA producer: 128B-swizzled 128x64 (A) and bn x 64 (B) BF16 tiles
//               into a 4-stage shared-memory ring (full/empty mbarriers);
//   warp 1      allocates 256 TMEM columns; one thread issues tcgen05.mma
//               (kind::f16, M=128, N=bn, K=16) and tcgen05.commit to free stages;
//   warps 2..5  epilogue: tcgen05.ld 32x32b from their TMEM lane quarter and
//               scatter alpha*acc + beta*C through the output offset tables.
// The K loop runs three segments over the packed operands (hi*hi, hi*lo,
// lo*hi).  Every mbarrier wait is bounded (~2 s): on expiry the kernel sets an
// error word, lets its in-flight TMA copies land, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "gemm_tc.h"

namespace scess {

namespace {

constexpr int TC_BM = 128;
constexpr int TC_BK = 64;  // 64 BF16 = 128 B = one SWIZZLE_128B row
constexpr int TC_STAGES = 4;
constexpr int TC_MAX_BN = 256;
constexpr int TC_THREADS = 192;
constexpr uint32_t A_STAGE_BYTES = TC_BM * TC_BK * 2;      // 16 KiB
constexpr uint32_t B_STAGE_BYTES = TC_MAX_BN * TC_BK * 2;  // 32 KiB
constexpr uint32_t TMEM_COLS = 256;
constexpr size_t TC_SMEM_BYTES = 1024 /*align slack*/ + TC_STAGES * (A_STAGE_BYTES + B_STAGE_BYTES) +
                                 (2 * TC_STAGES + 1) * 8 + 8 + TC_MAX_BN * 8;

enum : unsigned { ERR_FULL_WAIT = 1, ERR_EMPTY_WAIT = 2, ERR_ACCUM_WAIT = 3 };

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false (and the error word set) after ~2^32 cycles or when
// another role of the CTA already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned *err,
                                          unsigned code) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (unsigned spin = 1;; spin++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((spin & 1023u) == 0) {
      if (*(volatile unsigned *)err) return false;
      if (clock64() - t0 > (1ll << 32)) {
        atomicCAS(err, 0u, code);
        return false;
      }
    }
  }
}

// Bounded wait that ignores the error word: used to let issued TMA copies land
// before the CTA exits (returns after ~2^32 cycles at the latest).
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1ll << 32)) return;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// core-matrix groups 1024 B apart (SBO), descriptor version 1 (sm_100 family).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;             // version
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D=F32, A=B=BF16, both K-major.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
  int rowA0, rowB0, M, N;
  int nkb;           // K blocks (of 64) per segment
  int nseg;          // 1 or 3
  int kb_per_split;  // K blocks per split (blockIdx.z)
  int bn;            // tile width, multiple of 16, <= 256
  int Kpad;          // lo offset in the packed rows
  float *partial;    // split-K partials (nullptr: direct epilogue)
  int64_t part_stride;
  unsigned *err;
};

__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   TcOut out, TcArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *As = smem;
  uint8_t *Bs = smem + TC_STAGES * A_STAGE_BYTES;
  uint64_t *full = (uint64_t *)(Bs + TC_STAGES * B_STAGE_BYTES);
  uint64_t *empty = full + TC_STAGES;
  uint64_t *accum = empty + TC_STAGES;
  uint32_t *tmem_slot = (uint32_t *)(accum + 1);
  int64_t *colOff = (int64_t *)(tmem_slot + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * a.bn;
  const int kb0 = blockIdx.z * a.kb_per_split;
  const int kb1 = min(a.nkb, kb0 + a.kb_per_split);
  const int nk = kb1 - kb0;
  const int iters = a.nseg * nk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (warp >= 2 && !a.partial) {
    for (int c = threadIdx.x - 64; c < a.bn; c += 128) {
      const int n = n0 + c;
      colOff[c] = n < a.N ? out.baseC + out.colC[n] : -1;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0 && iters > 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
      int last[TC_STAGES];
      for (int s = 0; s < TC_STAGES; s++) last[s] = -1;
      const uint32_t bytes = A_STAGE_BYTES + (uint32_t)a.bn * TC_BK * 2;
      for (int it = 0; it < iters; it++) {
        const int s = it % TC_STAGES;
        const uint32_t ph = (uint32_t)(it / TC_STAGES) & 1u;
        if (!mbar_wait(&empty[s], ph ^ 1u, a.err, ERR_EMPTY_WAIT)) break;
        const int seg = it / nk;
        const int kb = kb0 + it % nk;
        const int xa = (seg == 2 ? a.Kpad : 0) + kb * TC_BK;
        const int xb = (seg == 1 ? a.Kpad : 0) + kb * TC_BK;
        mbar_expect_tx(&full[s], bytes);
        tma_load_2d(As + s * A_STAGE_BYTES, &tmA, xa, a.rowA0 + m0, &full[s]);
        tma_load_2d(Bs + s * B_STAGE_BYTES, &tmB, xb, a.rowB0 + n0, &full[s]);
        last[s] = it;
      }
      // Let every issued copy land before the CTA may exit.
      for (int s = 0; s < TC_STAGES; s++)
        if (last[s] >= 0) mbar_drain(&full[s], (uint32_t)(last[s] / TC_STAGES) & 1u);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(TC_BM, a.bn);
      for (int it = 0; it < iters; it++) {
        const int s = it % TC_STAGES;
        const uint32_t ph = (uint32_t)(it / TC_STAGES) & 1u;
        if (!mbar_wait(&full[s], ph, a.err, ERR_FULL_WAIT)) break;
        tc_fence_after();
        const uint32_t abase = smem_u32(As + s * A_STAGE_BYTES);
        const uint32_t bbase = smem_u32(Bs + s * B_STAGE_BYTES);
#pragma unroll
        for (int k = 0; k < TC_BK / 16; k++) {
          mma_bf16(tmem, sw128_desc(abase + 32 * k), sw128_desc(bbase + 32 * k), idesc,
                   (it > 0 || k > 0) ? 1u : 0u);
        }
        mma_commit(&empty[s]);
      }
      mma_commit(accum);
    }
  } else {
    const int q = warp & 3;
    const int row = 32 * q + lane;
    const int m = m0 + row;
    const bool ok = mbar_wait(accum, 0, a.err, ERR_ACCUM_WAIT);
    tc_fence_after();
    const bool good = ok && (*(volatile unsigned *)a.err == 0) && iters > 0;
    if (good) {
      int64_t rowOff = 0;
      if (!a.partial && m < a.M) rowOff = out.rowC[m];
      for (int c = 0; c < a.bn; c += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c, v);
        if (m < a.M) {
          if (a.partial) {
            float *P = a.partial + (int64_t)blockIdx.z * a.part_stride;
#pragma unroll
            for (int j = 0; j < 16; j++) {
              const int n = n0 + c + j;
              if (n < a.N) P[(int64_t)m + (int64_t)a.M * n] = v[j];
            }
          } else if (out.fp32) {
            float *C = (float *)out.C;
#pragma unroll
            for (int j = 0; j < 16; j++) {
              const int64_t co = colOff[c + j];
              if (co >= 0) {
                const int64_t off = rowOff + co;
                float val = (float)out.alpha * v[j];
                if (out.beta != 0.0) val += (float)out.beta * C[off];
                C[off] = val;
              }
            }
          } else {
            double *C = (double *)out.C;
#pragma unroll
            for (int j = 0; j < 16; j++) {
              const int64_t co = colOff[c + j];
              if (co >= 0) {
                const int64_t off = rowOff + co;
                double val = out.alpha * (double)v[j];
                if (out.beta != 0.0) val += out.beta * C[off];
                C[off] = val;
              }
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

__global__ void tc_reduce_kernel(TcOut out, int64_t M, int64_t N, int splits,
                                 const float *__restrict__ partial) {
  const int64_t MN = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; z++) s += (double)partial[(int64_t)z * MN + e];
    const int64_t m = e % M, n = e / M;
    const int64_t off = out.baseC + out.rowC[m] + out.colC[n];
    if (out.fp32) {
      float *C = (float *)out.C;
      double val = out.alpha * s;
      if (out.beta != 0.0) val += out.beta * (double)C[off];
      C[off] = (float)val;
    } else {
      double *C = (double *)out.C;
      double val = out.alpha * s;
      if (out.beta != 0.0) val += out.beta * C[off];
      C[off] = val;
    }
  }
}

// Gathers rows x K FP64 values through offset tables into BF16 hi/lo rows.
__global__ void __launch_bounds__(256) pack_split_kernel(
    const double *__restrict__ src, const int64_t *__restrict__ rowOff, int64_t rows,
    const int64_t *__restrict__ kOff, int64_t K, int unitK, __nv_bfloat16 *__restrict__ dst,
    int64_t Kpad) {
  __shared__ double tile[32][65];
  __shared__ int64_t sr[32], sk[64];
  const int t = threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 64;
  if (t < 32) sr[t] = (r0 + t < rows) ? rowOff[r0 + t] : -1;
  else if (t < 96) sk[t - 32] = (k0 + t - 32 < K) ? kOff[k0 + t - 32] : -1;
  __syncthreads();
#pragma unroll
  for (int p = 0; p < 8; p++) {
    int rr, kk;
    if (unitK) { kk = t & 63; rr = (t >> 6) + 4 * p; }
    else { rr = t & 31; kk = (t >> 5) + 8 * p; }
    const int64_t ro = sr[rr], ko = sk[kk];
    tile[rr][kk] = (ro >= 0 && ko >= 0) ? src[ro + ko] : 0.0;
  }
  __syncthreads();
  const int rr = t >> 3, ch = t & 7;
  __align__(16) __nv_bfloat16 hi[8];
  __align__(16) __nv_bfloat16 lo[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const double x = tile[rr][ch * 8 + j];
    const __nv_bfloat16 h = __double2bfloat16(x);
    hi[j] = h;
    lo[j] = __double2bfloat16(x - (double)__bfloat162float(h));
  }
  const int64_t base = (r0 + rr) * 2 * Kpad + k0 + ch * 8;
  *reinterpret_cast<uint4 *>(dst + base) = *reinterpret_cast<const uint4 *>(hi);
  *reinterpret_cast<uint4 *>(dst + base + Kpad) = *reinterpret_cast<const uint4 *>(lo);
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!fn) throw Error(SCESS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  return fn;
}

CUtensorMap make_map(const __nv_bfloat16 *base, int64_t rows_pad, int64_t Kpad, int box_rows) {
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  cuuint64_t dims[2] = {(cuuint64_t)(2 * Kpad), (cuuint64_t)rows_pad};
  cuuint64_t strides[1] = {(cuuint64_t)(2 * Kpad * 2)};
  cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = get_encode()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides,
                            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(SCESS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

}  // namespace

int TcEngine::tile_n(int64_t N) {
  const int64_t ntn = ceil_div(N, TC_MAX_BN);
  return (int)round_up(ceil_div(N, ntn), 16);
}

CUtensorMap TcEngine::map_of(const Packed &p, int box_rows) {
  return make_map(p.p(), p.rows_pad, p.Kpad, box_rows);
}

void tc_gemm_launch_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t rowA0,
                         int64_t M, int64_t rowB0, int64_t N, int bn, const TcOut &out, int nseg,
                         int splits, float *partial, unsigned *err, cudaStream_t stream) {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)TC_SMEM_BYTES);
  });
  if (M <= 0 || N <= 0) return;
  if (Kpad % TC_BK != 0 || Kpad <= 0) throw Error(SCESS_ERR_INVALID, "tc_gemm: Kpad % 64");
  if (M > INT32_MAX || N > INT32_MAX || rowA0 + M > INT32_MAX || rowB0 + N > INT32_MAX ||
      2 * Kpad > INT32_MAX)
    throw Error(SCESS_ERR_INVALID, "tc_gemm: dimension too large");
  if (bn % 16 != 0 || bn < 16 || bn > TC_MAX_BN) throw Error(SCESS_ERR_INVALID, "tc_gemm: bad bn");
  const int nkb = (int)(Kpad / TC_BK);
  if (splits < 1) splits = 1;
  if (splits > nkb) splits = nkb;
  const int kbs = (int)ceil_div(nkb, splits);
  splits = (int)ceil_div(nkb, kbs);
  TcArgs a;
  a.rowA0 = (int)rowA0;
  a.rowB0 = (int)rowB0;
  a.M = (int)M;
  a.N = (int)N;
  a.nkb = nkb;
  a.nseg = nseg;
  a.kb_per_split = kbs;
  a.bn = bn;
  a.Kpad = (int)Kpad;
  a.partial = splits > 1 ? partial : nullptr;
  a.part_stride = M * N;
  a.err = err;
  if (splits > 1 && !partial) throw Error(SCESS_ERR_INVALID, "tc_gemm: split-K needs partials");
  dim3 grid((unsigned)ceil_div(N, bn), (unsigned)ceil_div(M, TC_BM), (unsigned)splits);
  tc_gemm_kernel<<<grid, TC_THREADS, TC_SMEM_BYTES, stream>>>(ma, mb, out, a);
  SCESS_CHECK_LAUNCH();
  if (splits > 1) {
    const int64_t MN = M * N;
    tc_reduce_kernel<<<(unsigned)std::min<int64_t>(ceil_div(MN, 256), 8192), 256, 0, stream>>>(
        out, M, N, splits, partial);
    SCESS_CHECK_LAUNCH();
  }
}

void tc_gemm_launch(const __nv_bfloat16 *A, int64_t a_rows_pad, const __nv_bfloat16 *B,
                    int64_t b_rows_pad, int64_t Kpad, int64_t rowA0, int64_t M, int64_t rowB0,
                    int64_t N, const TcOut &out, int nseg, int splits, float *partial,
                    unsigned *err, cudaStream_t stream) {
  if (M <= 0 || N <= 0) return;
  const int bn = TcEngine::tile_n(N);
  const CUtensorMap ma = make_map(A, a_rows_pad, Kpad, TC_BM);
  const CUtensorMap mb = make_map(B, b_rows_pad, Kpad, bn);
  tc_gemm_launch_maps(ma, mb, Kpad, rowA0, M, rowB0, N, bn, out, nseg, splits, partial, err, stream);
}

void TcEngine::gemm_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t rowA0,
                         int64_t M, int64_t rowB0, int64_t N, const TcOut &out, int nseg,
                         cudaStream_t stream) {
  tc_gemm_launch_maps(ma, mb, Kpad, rowA0, M, rowB0, N, tile_n(N), out, nseg, 1, nullptr,
                      err_.as<unsigned>(), stream ? stream : ctx_.stream);
}

// ---------------------------------------------------------------------------------------------

TcEngine::TcEngine(Ctx &ctx) : ctx_(ctx) {
  err_.alloc(sizeof(unsigned) * 4);
  SCESS_CUDA(cudaMemsetAsync(err_.as<void>(), 0, sizeof(unsigned) * 4, ctx_.stream));
}

TcEngine::~TcEngine() = default;

bool TcEngine::worth_it(const EinsumPlan &pl) {
  const int64_t mx = std::max(pl.M, pl.N), mn = std::min(pl.M, pl.N);
  return mx >= 64 && mn >= 16 && pl.K >= 8 && 2.0 * pl.M * pl.N * pl.K >= 2.0e7;
}

void TcEngine::pack(const double *src, const int64_t *rowOff, int64_t rows, const int64_t *kOff,
                    int64_t K, bool unitK, int64_t row_align, Packed &out) {
  const int64_t Kpad = round_up(std::max<int64_t>(K, 1), TC_BK);
  const int64_t rows_pad = round_up(std::max<int64_t>(rows, 1), std::max<int64_t>(row_align, 32));
  const size_t bytes = (size_t)rows_pad * 2 * Kpad * sizeof(__nv_bfloat16);
  if (out.mem.bytes() < bytes) {
    ctx_.sync();
    out.mem.alloc(bytes);
  }
  out.rows = rows;
  out.rows_pad = rows_pad;
  out.K = K;
  out.Kpad = Kpad;
  dim3 grid((unsigned)(Kpad / 64), (unsigned)(rows_pad / 32));
  pack_split_kernel<<<grid, 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K, unitK ? 1 : 0,
                                                   out.p(), Kpad);
  SCESS_CHECK_LAUNCH();
}

void TcEngine::gemm(const Packed &A, int64_t rowA0, int64_t M, const Packed &B, int64_t rowB0,
                    int64_t N, const TcOut &out, int nseg, int force_splits) {
  if (A.Kpad != B.Kpad) throw Error(SCESS_ERR_INVALID, "tc gemm: K mismatch");
  const int nkb = (int)(A.Kpad / TC_BK);
  int splits = force_splits;
  if (splits <= 0) {
    const int64_t ntn = ceil_div(N, TC_MAX_BN);
    const int64_t tiles = ceil_div(M, TC_BM) * ntn;
    splits = 1;
    if (tiles < kNumSMs) {
      splits = (int)std::min<int64_t>(ceil_div(kNumSMs, tiles), std::max(1, nkb / 4));
      while (splits > 1 && (int64_t)splits * M * N > (int64_t(256) << 20)) splits--;
    }
  }
  float *partial = nullptr;
  if (splits > 1) {
    const size_t need = (size_t)splits * M * N * sizeof(float);
    if (partial_.bytes() < need) {
      ctx_.sync();
      partial_.alloc(need);
    }
    partial = partial_.as<float>();
  }
  tc_gemm_launch(A.p(), A.rows_pad, B.p(), B.rows_pad, A.Kpad, rowA0, M, rowB0, N, out, nseg,
                 splits, partial, err_.as<unsigned>(), ctx_.stream);
}

void TcEngine::check_error() {
  unsigned h = 0;
  SCESS_CUDA(cudaMemcpyAsync(&h, err_.as<void>(), sizeof(unsigned), cudaMemcpyDeviceToHost,
                             ctx_.stream));
  ctx_.sync();
  if (h != 0) {
    SCESS_CUDA(cudaMemsetAsync(err_.as<void>(), 0, sizeof(unsigned), ctx_.stream));
    throw Error(SCESS_ERR_CUDA, "tensor-core pipeline wait expired (code " + std::to_string(h) + ")");
  }
}

void TcEngine::contract(const EinsumPlan &pl, double alpha, const double *A, const double *B,
                        double beta, double *C, bool constA, bool constB) {
  // Put the longer output side on the 128-row MMA dimension.
  const bool swap = pl.M < 64 && pl.N >= 64;
  const int64_t *rowX = swap ? pl.d_colB : pl.d_rowA, *kX = swap ? pl.d_kB : pl.d_kA;
  const int64_t *rowY = swap ? pl.d_rowA : pl.d_colB, *kY = swap ? pl.d_kA : pl.d_kB;
  const double *X = swap ? B : A, *Y = swap ? A : B;
  const bool cX = swap ? constB : constA, cY = swap ? constA : constB;
  const bool uX = swap ? pl.bUnitK : pl.aUnitK, uY = swap ? pl.aUnitK : pl.bUnitK;
  const int64_t MX = swap ? pl.N : pl.M, NY = swap ? pl.M : pl.N;

  auto get = [&](const double *src, const int64_t *rows, int64_t nrows, const int64_t *ks,
                 bool unitK, bool isConst, const char *tag, Packed &tmp) -> const Packed & {
    if (!isConst) {
      pack(src, rows, nrows, ks, pl.K, unitK, TC_BM, tmp);
      return tmp;
    }
    std::string key = pl.key + tag + std::to_string((uintptr_t)src);
    auto it = cache_.find(key);
    if (it != cache_.end()) return *it->second;
    auto pk = std::make_unique<Packed>();
    pack(src, rows, nrows, ks, pl.K, unitK, TC_BM, *pk);
    auto &ref = *pk;
    cache_.emplace(key, std::move(pk));
    return ref;
  };
  const Packed &PX = get(X, rowX, MX, kX, uX, cX, swap ? "#B" : "#A", tmpA_);
  const Packed &PY = get(Y, rowY, NY, kY, uY, cY, swap ? "#A" : "#B", tmpB_);
  TcOut o;
  o.C = C;
  o.fp32 = 0;
  o.rowC = swap ? pl.d_colC : pl.d_rowC;
  o.colC = swap ? pl.d_rowC : pl.d_colC;
  o.alpha = alpha;
  o.beta = beta;
  gemm(PX, 0, MX, PY, 0, NY, o, 3);
}

}  // namespace scess
