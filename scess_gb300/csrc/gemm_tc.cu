// tcgen05 / TMEM / TMA tensor-core GEMM for sm_103a (split 16-bit hi+lo, FP32 accumulate).
//
// A persistent CTA per SM walks work units (problem, 128 x BN tile, K range):
//   warp 0      TMA producer: 128B-swizzled 128x64 (A) and BNx64 (B) tiles of
//               the hi and lo halves into a shared-memory ring (full/empty
//               mbarriers; 3 stages at BN = 128, 2 at BN = 256);
//   warp 1      allocates all 512 TMEM columns (512 / BN accumulators); one
//               thread issues tcgen05.mma (kind::f16, M=128, N<=BN, K=16) and
//               tcgen05.commit to free stages and hand accumulators over;
//   the rest    epilogue warps (one warpgroup per 128 columns): tcgen05.ld
//               32x32b from their TMEM lane quarter every K block (or every
//               second), FP32 accumulation in registers, and the scatter of
//               alpha*acc + beta*C through the output offset tables.
// The K loop runs three products over the packed operands (hi*hi, hi*lo,
// lo*hi).  Every mbarrier wait is bounded (~2 s): on expiry the kernel sets an
// error word, lets its in-flight TMA copies land, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cuda_fp16.h>

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "gemm_tc.h"
#include "mbarrier.cuh"

namespace scess {

namespace {

constexpr int TC_BM = 128;
constexpr int TC_BK = 64;  // K padding of the packs; 64 x 16 bit = 128 B = one SWIZZLE_128B row

enum : unsigned { ERR_FULL_WAIT = 1, ERR_EMPTY_WAIT = 2, ERR_ACCUM_WAIT = 3 };

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Two-SM (cluster pair) forms.  The pair's even CTA issues the MMAs; its
// shared-memory barriers count both CTAs' copies and both CTAs' drains.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t nclusters_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of the same shared-memory object in the pair's rank-0 CTA.
__device__ __forceinline__ uint32_t leader_addr(const void *p) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(r) : "r"(smem_u32(p)));
  return r;
}
// TMA load into this CTA's shared memory whose completion is counted on a
// barrier of either CTA of the pair (cluster address).
__device__ __forceinline__ void tma_load_2d_pair(void *dst, const CUtensorMap *tm, int x, int y,
                                                 uint32_t bar_cluster) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], "
      "[%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(bar_cluster)
      : "memory");
}
// Arrival on a barrier of either CTA of the pair.  Release at CTA scope: it
// only has to follow this thread's completed TMEM loads (tcgen05.wait::ld);
// a cluster-scope release would also wait for the thread's earlier global
// stores to be acknowledged.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cta.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Fire-and-forget FP32 reduction into global memory (an L2 atomic) of four
// consecutive floats at a 16-byte aligned address.
__device__ __forceinline__ void red_add_v4(float *p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}


// Shared-memory matrix descriptor of a K-major operand whose rows are SWZ
// bytes (one swizzle span: 128 or 64): 8-row core-matrix groups 8 x SWZ bytes
// apart (SBO), descriptor version 1 (sm_100 family), layout type 2
// (SWIZZLE_128B) or 4 (SWIZZLE_64B).  The leading byte offset is unused for
// swizzled K-major operands (one MMA's K = 16 x 16 bit = 32 B stays inside a row).
template <int SWZ>
__device__ __forceinline__ uint64_t sw_desc(uint32_t saddr) {
  static_assert(SWZ == 128 || SWZ == 64, "swizzle span");
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused)
  d |= (uint64_t)((8 * SWZ) >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;                   // version
  d |= (uint64_t)(SWZ == 128 ? 2 : 4) << 61;
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D=F32, A=B=BF16 (fmt 1) or
// F16 (fmt 0), both K-major; N>>3 at bits 17-22, M>>4 at bits 24-28.
__device__ __forceinline__ uint32_t idesc_f16kind(int M, int N, uint32_t ab_fmt) {
  return (1u << 4) | (ab_fmt << 7) | (ab_fmt << 10) | ((uint32_t)(N >> 3) << 17) |
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

// M = 256 over the pair: A rows 0-127 from this CTA's shared memory, 128-255
// from the peer's at the same offset; B columns split likewise (N/2 each); D
// rows 0-127 in this SM's TMEM, 128-255 in the peer's.
__device__ __forceinline__ void mma2_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
// Arrive on the barrier at this offset in both CTAs of the pair once the
// issued MMAs have completed.
__device__ __forceinline__ void mma2_commit_both(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"((uint16_t)3)
      : "memory");
}
__device__ __forceinline__ void mma2_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Asynchronous form: the 16 registers are valid after tmem_wait16 on them
// (the wait takes them as operands, so no use can be scheduled before it).
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// 16x256b shape, 4 repetitions: thread t gets TMEM lanes base + t/4 (r[4j],
// r[4j+1]) and base + 8 + t/4 (r[4j+2], r[4j+3]), columns 8j + 2 (t % 4) and
// the next, j = 0..3 (the accumulator fragment of an m16n8 tile per repetition).
__device__ __forceinline__ void tmem_ld16x256b_x4_async(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.16x256b.x4.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait16(uint32_t *r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
               :
               : "memory");
}

// TMEM loads (16 columns each) issued per wait in the drain.
#ifndef SCESS_TC_LDB
#define SCESS_TC_LDB 1
#endif

// K segment of a tensor-core problem: operand maps, K blocks, lo offset and the
// first A/B row of problem (y, z) of group g: row0[g] + y * row_y[g] + z * row_z[g].
struct TcSegArgs {
  int mapA, mapB;
  int nkb;   // K blocks of this segment
  int bk;    // their width: the kernel's BK, or 32 (64-byte swizzle, half-filled stages)
  int kpad;  // lo offset in the packed rows (elements)
  int negA;  // negate this segment's products
  int64_t rowA0[3], rowAy[3], rowAz[3], rowB0[3], rowBy[3], rowBz[3];
};

struct TcMaps {
  CUtensorMap m[6];
};

struct TcArgs {
  int M, N;
  int tiles_m, tiles_n;
  int ny, nz, ng;    // problems: (y, z, g) in [0, ny) x [0, nz) x [0, ng)
  int nseg;          // K segments (<= 4)
  int kb_total;      // sum of the segments' K blocks
  int kb_per_split;  // K blocks per work unit (split-K when < kb_total)
  int splits;
  int f16;           // operands are FP16 (else BF16)
  int split3;        // three hi/lo products (else hi*hi only)
  int kbd;           // K blocks accumulated in one TMEM buffer per drain (1 or 2)
  TcSegArgs seg[4];
  int64_t cy[3], cz[3];  // output offset of problem (y, z, g): y * cy[g] + z * cz[g] + cg[g]
  int64_t cg[3];
  const int64_t *rowCg[3], *colCg[3];  // per-group output tables (null: TcOut's)
  int tri[3];                          // group g keeps only the problems with y >= z (ny == nz)
  int gstart[4];                       // first problem index of each group (gstart[ng] = total)
  int stcol[3];                        // group stores along columns (FP32, beta = 0)
  int stvec[3];                        // ... in contiguous aligned quads of columns
  float *partial;    // split-K partials (nullptr: direct epilogue)
  int64_t part_stride;
  unsigned *err;
  long long wait_cycles;  // bound of every pipeline wait (clock64 cycles)
  int withhold_first;     // diagnostics: the producer never fills its first stage
};

// Persistent tcgen05 GEMM over work units (problem, 128 x 128 output tile, K range).
//   warp 0     TMA producer: per 64-wide K block one smem stage holding A_hi,
//              A_lo, B_hi, B_lo (128 rows x 128 B each, 128B swizzle);
//   warp 1     TMEM owner + MMA issuer: the block's products lo*hi, hi*lo,
//              hi*hi (4 x K=16 each) go into one of four 128-column TMEM
//              buffers, starting from zero, then tcgen05.commit;
//   warps 2-5  drain each buffer into an FP32 register accumulator (one row
//              per thread, round-to-nearest adds) and, after the unit's last K
//              block, scatter alpha*acc + beta*C through the offset tables.
// Draining every K block (kbd = 1) bounds the truncating accumulation inside
// TMEM to the 12 products of one block, so the result's error does not grow
// with K; kbd = 2 drains every second block (half the drains, about twice the
// per-element rounding error, still K-independent).
// A problem's K range may span several segments with different operands
// (up to 4), each optionally negated through the instruction descriptor.
constexpr int V2_BN = 128;  // tile width of the einsum launches

// Shape of a kernel instantiation by tile width BN (128 or 256):
//   BN = 128: K blocks of 64 (128-byte rows, SWIZZLE_128B), 3 stages of
//             64 KiB, four 128-column TMEM accumulators, 192 threads (warps
//             2-5 drain and store);
//   BN = 256: K blocks of 64 in 2 stages of 96 KiB, or of 32 (64-byte rows,
//             SWIZZLE_64B) in 4 stages of 48 KiB (the same 192 KiB, three
//             stages in flight while one is consumed); two 256-column
//             accumulators, 384 threads (warps 2-3 idle, warps 4-7 / 8-11
//             drain and store columns 0-127 / 128-255).  With more than one
//             warp per scheduler beside the epilogue the block is capped at
//             168 registers a thread, so the warpgroups rebalance with
//             setmaxnreg: 56 for warps 0-3, 224 for the epilogue (3 x 168 =
//             56 + 2 x 224 per scheduler).
//   PAIR:     BN = 256, BK = 64 on a cluster pair (M = 256 per unit, 128 rows
//             a CTA): each CTA stages its A rows and half of the B columns,
//             64 KiB a stage, 3 stages.
// Every epilogue thread holds 128 columns of one row.
template <int BN, int BK_, bool PAIR = false>
struct TcShape {
  static_assert((BN == 128 && BK_ == 64) || (BN == 256 && (BK_ == 64 || BK_ == 32)), "shape");
  static_assert(!PAIR || (BN == 256 && BK_ == 64), "pair shape");
  static constexpr int BK = BK_;                   // K per stage (16-bit elements)
  static constexpr int SWZ = 2 * BK;               // row bytes = swizzle span
  static constexpr int STAGES = PAIR ? 3 : (BN == 128 ? 3 : (BK == 64 ? 2 : 4));
  static constexpr int BM = PAIR ? 2 * TC_BM : TC_BM;  // rows of a unit
  static constexpr int BNL = PAIR ? BN / 2 : BN;       // B rows staged by one CTA
  static constexpr int NBUF = 512 / BN;
  static constexpr int EPI0 = BN == 256 ? 4 : 2;   // first epilogue warp
  static constexpr int NEPI = BN / 32;              // epilogue warps
  static constexpr int THREADS = 32 * (EPI0 + NEPI);
  static constexpr int CH = BN == 256 ? 16 : 32;    // columns per staged chunk
  static constexpr uint32_t A_BYTES = (uint32_t)TC_BM * BK * 2;
  static constexpr uint32_t B_BYTES = (uint32_t)BNL * BK * 2;
  static constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr uint32_t TMEM_COLS = 512;
  // 1 KiB alignment slack in front, the barriers behind the stages, and 1 KiB
  // of tail slack so that no descriptor-addressed read can leave the allocation
  static constexpr size_t SMEM_BYTES =
      1024 + STAGES * STAGE_BYTES + (2 * STAGES + 2 * NBUF + 1) * 8 + 8 + 1024;
};
constexpr int kEpiRegs256 = 224, kCtlRegs256 = 56, kLaunchRegs256 = 168;

__device__ __forceinline__ void seg_of(const TcArgs &a, int kb, int &s, int &lkb) {
  s = 0;
  lkb = kb;
  while (s < a.nseg - 1 && lkb >= a.seg[s].nkb) {
    lkb -= a.seg[s].nkb;
    s++;
  }
}

// Persistent tcgen05 GEMM over work units (problem, 128 x BN output tile, K range).
//   warp 0     TMA producer: per 64-wide K block one smem stage holding A_hi,
//              B_hi, A_lo, B_lo (128 / BN rows x 128 B, 128B swizzle);
//   warp 1     TMEM owner + MMA issuer: the block's products lo*hi, hi*lo,
//              hi*hi (4 x K=16 each) go into one of the BN-column TMEM
//              buffers, starting from zero, then tcgen05.commit;
//   epilogue   drain each buffer into an FP32 register accumulator (one row,
//              128 columns per thread, round-to-nearest adds) and, after the
//              unit's last K block, scatter alpha*acc + beta*C through the
//              offset tables.
// Draining every K block (kbd = 1) bounds the truncating accumulation inside
// TMEM to the 12 products of one block, so the result's error does not grow
// with K; kbd = 2 drains every second block (half the drains, about twice the
// per-element rounding error, still K-independent).
// A problem's K range may span several segments with different operands
// (up to 4), each optionally negated through the instruction descriptor.
// the MMA of the kernel's form (one CTA, or the pair)
#define MMA_(...)                         \
  do {                                    \
    if constexpr (PAIR) mma2_bf16(__VA_ARGS__); \
    else mma_bf16(__VA_ARGS__);           \
  } while (0)

template <int BN, int BK, bool PAIR = false>
__global__ void __launch_bounds__(TcShape<BN, BK, PAIR>::THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ TcMaps maps, TcOut out, TcArgs a) {
  using SH = TcShape<BN, BK, PAIR>;
  constexpr int STAGES = SH::STAGES, NBUF = SH::NBUF, HC = 128;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + STAGES * SH::STAGE_BYTES);
  uint64_t *empty = full + STAGES;
  uint64_t *tfull = empty + STAGES;      // [NBUF]
  uint64_t *tempty = tfull + NBUF;       // [NBUF]
  uint64_t *done = tempty + NBUF;        // [1]
  uint32_t *tmem_slot = (uint32_t *)(done + 1);
  // Column offsets of the current unit.  A statically declared shared array:
  // the compiler then knows these loads cannot alias the global stores of the
  // scatter and batches them (through a generic pointer every load would wait
  // for the previous store).
  __shared__ int64_t colOff[BN];
  __shared__ int64_t rowOffS[BN / 128][TC_BM];        // row offsets of a column-stored unit
  // chunk of such a unit; row pitch 129 (CH = 32) or 130 (CH = 16, two rows a
  // warp step) keeps the column-wise reads free of bank conflicts
  __shared__ float stage[BN / 128][SH::CH][TC_BM + (SH::CH == 16 ? 2 : 1)];
  // Output scaling, once per CTA: alpha / (sA sB) with power-of-two pack
  // scales sA, sB.  FP32 outputs multiply by it in FP32; FP64 outputs multiply
  // by the user's alpha in FP32 and apply 2^-log2(sA sB) to the exponent field
  // (exact, no FP64 arithmetic per element).
  __shared__ double s_alpha;
  __shared__ float s_falpha, s_fuser;
  __shared__ int s_shift, s_shift_ok;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles = a.tiles_m * a.tiles_n;
  const int nprob = a.gstart[a.ng];
  const int units = tiles * nprob * a.splits;
  // work distribution: per CTA, or per cluster pair (rank 0 issues the MMAs)
  const int rank = PAIR ? (int)cluster_rank() : 0;
  const int wid = PAIR ? (int)cluster_id_x() : (int)blockIdx.x;
  const int nwork = PAIR ? (int)nclusters_x() : (int)gridDim.x;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < NBUF; b++) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], SH::NEPI * (PAIR ? 2 : 1));  // one arrival per epilogue warp (of the pair)
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    double sc = 1.0;
    if (out.scaleA) sc *= *out.scaleA;
    if (out.scaleB) sc *= *out.scaleB;
    s_alpha = out.alpha / sc;
    s_falpha = (float)(out.alpha / sc);
    s_fuser = (float)out.alpha;
    int e = 0;
    const double f = frexp(sc, &e);  // sc = 0.5 * 2^e exactly for a power of two
    s_shift = 1 - e;
    s_shift_ok = (f == 0.5 && e > -400 && e < 400) ? 1 : 0;
  }
  if (warp == 1) {
    if constexpr (PAIR) {  // one warp of each CTA of the pair, collectively
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(tmem_slot)),
                   "r"(SH::TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(tmem_slot)),
                   "r"(SH::TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
  }
  tc_fence_before();
  __syncthreads();
  // the peer's barriers are initialised before any copy or arrival targets them
  if constexpr (PAIR) cluster_sync_all();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // the stream's next kernel may be scheduled once every CTA is here (it waits
  // for this grid's completion before it reads what this grid writes)
  if (threadIdx.x == 0) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

  // The CTA's it-th unit: round it of a round-robin over the grid whose odd
  // rounds swap neighbouring CTAs, so that with an even grid and two column
  // tiles per problem (a full one and a narrower remainder) every CTA gets
  // both kinds in turn instead of always the same one.
  auto unit_at = [&](int it) -> int {
    int b = wid;
    if (it & 1) {
      const int p = b ^ 1;
      if (p < nwork) b = p;
    }
    return it * nwork + b;
  };
  // unit -> (tile m, tile n, problem y, z, g, K-block range)
  auto unit_coords = [&](int u, int &tm, int &tn, int &py, int &pz, int &pg, int &kb0, int &kb1) {
    const int tile = u % tiles;
    const int rest = u / tiles;
    const int q = rest % nprob;
    const int sp = rest / nprob;
    tn = tile % a.tiles_n;
    tm = tile / a.tiles_n;
    if constexpr (BN != 256) {  // (einsum launches: no triangular groups)
      py = q % a.ny;
      pz = (q / a.ny) % a.nz;
      pg = q / (a.ny * a.nz);
      kb0 = sp * a.kb_per_split;
      kb1 = min(a.kb_total, kb0 + a.kb_per_split);
      return;
    }
    pg = 0;
    while (pg + 1 < a.ng && q >= a.gstart[pg + 1]) pg++;
    const int lq = q - a.gstart[pg];
    if (a.tri[pg]) {  // lq = y (y + 1) / 2 + z, z <= y
      int y = (int)((sqrtf(8.0f * (float)lq + 1.0f) - 1.0f) * 0.5f);
      while (y * (y + 1) / 2 > lq) y--;
      while ((y + 1) * (y + 2) / 2 <= lq) y++;
      py = y;
      pz = lq - y * (y + 1) / 2;
    } else {
      py = lq % a.ny;
      pz = lq / a.ny;
    }
    kb0 = sp * a.kb_per_split;
    kb1 = min(a.kb_total, kb0 + a.kb_per_split);
  };

  if (warp < SH::EPI0) {  // control warps: TMA producer, MMA issuer (and idle warps)
    if constexpr (BN == 256) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kCtlRegs256));
  if (warp == 0) {
    if (lane == 0) {
      for (int i = 0; i < 6; i++)
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&maps.m[i]) : "memory");
      const uint32_t bytes = a.split3 ? SH::STAGE_BYTES : SH::A_BYTES + SH::B_BYTES;
      int g = 0;
      int last[STAGES];
      for (int s = 0; s < STAGES; s++) last[s] = -1;
      bool ok = true;
      for (int it = 0; it * nwork < units && ok; it++) {
        const int u = unit_at(it);
        if (u >= units) continue;
        int tm, tn, py, pz, pg, kb0, kb1;
        unit_coords(u, tm, tn, py, pz, pg, kb0, kb1);
        // pair: this CTA stages A rows 128 rank.. of the unit and B columns from
        // rank x (half the MMA width) on
        int boff = 0;
        if constexpr (PAIR) boff = rank * (min(BN, (a.N - tn * BN + 31) & ~31) / 2);
        for (int kb = kb0; kb < kb1; kb++, g++) {
          int sg, lkb;
          seg_of(a, kb, sg, lkb);
          const TcSegArgs &S = a.seg[sg];
          const int ya = (int)(S.rowA0[pg] + py * S.rowAy[pg] + pz * S.rowAz[pg]) + tm * SH::BM +
                         rank * TC_BM;
          const int yb = (int)(S.rowB0[pg] + py * S.rowBy[pg] + pz * S.rowBz[pg]) + tn * BN + boff;
          const int s = g % STAGES;
          const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, a.err, ERR_EMPTY_WAIT, a.wait_cycles)) { ok = false; break; }
          // diagnostics: the first stage is taken but never filled, so that the
          // MMA thread's bounded wait on it runs out (nothing is in flight there)
          if (a.withhold_first && g == 0) continue;
          uint8_t *st = smem + s * SH::STAGE_BYTES;
          const CUtensorMap *mA = &maps.m[S.mapA], *mB = &maps.m[S.mapB];
          // a 32-wide block of a segment in a 64-wide kernel fills half a stage
          const uint32_t sb = S.bk == SH::BK ? bytes : bytes / 2;
          const int x = lkb * S.bk;
          if constexpr (PAIR) {
            // both CTAs' copies complete on the rank-0 CTA's barrier
            const uint32_t fb = leader_addr(&full[s]);
            if (rank == 0) mbar_expect_tx(&full[s], 2 * sb);
            tma_load_2d_pair(st, mA, x, ya, fb);                                    // A hi
            tma_load_2d_pair(st + SH::A_BYTES, mB, x, yb, fb);                      // B hi
            if (a.split3) {
              tma_load_2d_pair(st + SH::A_BYTES + SH::B_BYTES, mA, S.kpad + x, ya, fb);      // A lo
              tma_load_2d_pair(st + 2 * SH::A_BYTES + SH::B_BYTES, mB, S.kpad + x, yb, fb);  // B lo
            }
          } else {
            mbar_expect_tx(&full[s], sb);
            tma_load_2d(st, mA, x, ya, &full[s]);                                  // A hi
            tma_load_2d(st + SH::A_BYTES, mB, x, yb, &full[s]);                    // B hi
            if (a.split3) {
              tma_load_2d(st + SH::A_BYTES + SH::B_BYTES, mA, S.kpad + x, ya, &full[s]);  // A lo
              tma_load_2d(st + 2 * SH::A_BYTES + SH::B_BYTES, mB, S.kpad + x, yb, &full[s]);  // B lo
            }
          }
          last[s] = g;
        }
      }
      // (pair: the rank-0 barriers also count the peer's copies; the peer
      // leaves only after the cluster barrier at the end, i.e. after this
      // drain, and after an error it first gives its last copies ~50 us)
      if (!PAIR || rank == 0) {
        for (int s = 0; s < STAGES; s++)
          if (last[s] >= 0) mbar_drain(&full[s], (uint32_t)(last[s] / STAGES) & 1u);
      } else if (!ok) {
        const long long t0 = clock64();
        while (clock64() - t0 < 100000) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && (!PAIR || rank == 0)) {  // (pair: the rank-0 CTA issues for both)
      int g = 0, c = 0;
      bool ok = true;
      for (int it = 0; it * nwork < units && ok; it++) {
        const int u = unit_at(it);
        if (u >= units) continue;
        int tm, tn, py, pz, pg, kb0, kb1;
        unit_coords(u, tm, tn, py, pz, pg, kb0, kb1);
        // MMA width: the tile's valid columns rounded up to 16 (M = 128 takes any
        // N = 16..256 in steps of 16; the MMA time scales with N); pair: to 32,
        // so that each CTA's half of B is a whole number of 16-row groups
        const int nvalid = PAIR ? min(BN, (a.N - tn * BN + 31) & ~31) : min(BN, (a.N - tn * BN + 15) & ~15);
        const uint32_t idesc = idesc_f16kind(SH::BM, nvalid, a.f16 ? 0u : 1u);
        for (int kb = kb0; kb < kb1; kb++, g++) {
          int sg, lkb;
          seg_of(a, kb, sg, lkb);
          const uint32_t id = idesc | (a.seg[sg].negA ? (1u << 13) : 0u);  // negate A
          const int s = g % STAGES;
          const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
          const int b = c % NBUF;
          const uint32_t bph = (uint32_t)(c / NBUF) & 1u;
          const bool first = (kb - kb0) % a.kbd == 0;
          const bool last = (kb - kb0) % a.kbd == a.kbd - 1 || kb == kb1 - 1;
          if (first && !mbar_wait(&tempty[b], bph ^ 1u, a.err, ERR_EMPTY_WAIT, a.wait_cycles)) { ok = false; break; }
          if (!mbar_wait(&full[s], ph, a.err, ERR_FULL_WAIT, a.wait_cycles)) { ok = false; break; }
          tc_fence_after();
          const uint32_t st = smem_u32(smem + s * SH::STAGE_BYTES);
          const uint32_t ahi = st, bhi = st + SH::A_BYTES;
          const uint32_t alo = st + SH::A_BYTES + SH::B_BYTES;
          const uint32_t blo = st + 2 * SH::A_BYTES + SH::B_BYTES;
          const uint32_t d = tmem + (uint32_t)(b * BN);
          uint32_t acc = first ? 0u : 1u;
          if (SH::BK == 64 && a.seg[sg].bk == 32) {
            // half-filled stage of a 32-wide segment: 64-byte rows, 64-byte swizzle
            if (a.split3) {
#pragma unroll
              for (int k = 0; k < 2; k++, acc = 1)
                MMA_(d, sw_desc<64>(alo + 32 * k), sw_desc<64>(bhi + 32 * k), id, acc);
#pragma unroll
              for (int k = 0; k < 2; k++)
                MMA_(d, sw_desc<64>(ahi + 32 * k), sw_desc<64>(blo + 32 * k), id, 1u);
            }
#pragma unroll
            for (int k = 0; k < 2; k++, acc = 1)
              MMA_(d, sw_desc<64>(ahi + 32 * k), sw_desc<64>(bhi + 32 * k), id, acc);
          } else {
            if (a.split3) {
#pragma unroll
              for (int k = 0; k < SH::BK / 16; k++, acc = 1)
                MMA_(d, sw_desc<SH::SWZ>(alo + 32 * k), sw_desc<SH::SWZ>(bhi + 32 * k), id, acc);
#pragma unroll
              for (int k = 0; k < SH::BK / 16; k++)
                MMA_(d, sw_desc<SH::SWZ>(ahi + 32 * k), sw_desc<SH::SWZ>(blo + 32 * k), id, 1u);
            }
#pragma unroll
            for (int k = 0; k < SH::BK / 16; k++, acc = 1)
              MMA_(d, sw_desc<SH::SWZ>(ahi + 32 * k), sw_desc<SH::SWZ>(bhi + 32 * k), id, acc);
          }
          if constexpr (PAIR) {
            mma2_commit_both(&empty[s]);
            if (last) mma2_commit_both(&tfull[b]);
          } else {
            mma_commit(&empty[s]);
            if (last) mma_commit(&tfull[b]);
          }
          if (last) c++;
        }
      }
      // every MMA issued above has completed once `done` fires
      if constexpr (PAIR) mma2_commit(done);
      else mma_commit(done);
      mbar_drain(done, 0);
    }
  }
  } else {  // epilogue warps
    if constexpr (BN == 256) asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kEpiRegs256));
    // a programmatic dependent launch (TcProblemSet::pdl) stores only after the
    // previous grid is complete and its writes are visible (no-op otherwise)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int q = warp & 3;
    const int row = 32 * q + lane;
    const int h = (warp - SH::EPI0) >> 2;                 // column half (BN = 256)
    const int et = threadIdx.x - 32 * SH::EPI0 - 128 * h;  // 0..127 within the half
    const int bar = 1 + h;                                // named barrier of the half
    int64_t *colH = colOff + HC * h;
    int c = 0;
    bool ok = true;
    for (int it = 0; it * nwork < units && ok; it++) {
      const int u = unit_at(it);
      if (u >= units) continue;
      int tm, tn, py, pz, pg, kb0, kb1;
      unit_coords(u, tm, tn, py, pz, pg, kb0, kb1);
      const int m = tm * SH::BM + rank * TC_BM + row;
      const int n0 = tn * BN + HC * h;
      asm volatile("bar.sync %0, 128;" ::"r"(bar) : "memory");  // previous unit's colOff reads done
      if (!a.partial) {
        const int nn = n0 + et;
        const int64_t *colT = a.colCg[pg] ? a.colCg[pg] : out.colC;
        colH[et] = nn < a.N ? out.baseC + py * a.cy[pg] + pz * a.cz[pg] + a.cg[pg] + colT[nn] : -1;
      }
      // issued now, used after the K loop: their latency hides behind the MMAs
      const int64_t *rowT = a.rowCg[pg] ? a.rowCg[pg] : out.rowC;
      const int64_t rowOff = (!a.partial && m < a.M) ? rowT[m] : 0;
      // Units whose output runs along pairs of columns (the (T) groups stored by
      // column in aligned quads): TMEM is drained in the 16x256b shape, so that
      // each thread holds column pairs of rows 32 q + 8 s + lane / 4 (s = 0..3)
      // and stores them straight from registers (no staging through shared memory).
      // beta = 1 (FP32 outputs stored along columns): the unit adds into C with
      // L2 reductions instead of storing
      const bool accum = out.beta == 1.0;
      const bool pc = BN == 256 && a.stvec[pg] && out.fp32 && (out.beta == 0.0 || accum) && !a.partial;
      const unsigned errv = *(volatile unsigned *)a.err;
      float acc[HC];
#pragma unroll
      for (int j = 0; j < HC; j++) acc[j] = 0.0f;
      // (two copies of the drain loop, one per TMEM load shape: one loop with
      // both shapes keeps the accumulators in local memory)
      if (pc) {
        for (int kb = kb0; kb < kb1; kb += a.kbd, c++) {
          const int b = c % NBUF;
          const uint32_t bph = (uint32_t)(c / NBUF) & 1u;
          if (!mbar_wait(&tfull[b], bph, a.err, ERR_ACCUM_WAIT, a.wait_cycles)) { ok = false; break; }
          tc_fence_after();
          const uint32_t t0 = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * BN + HC * h);
          // acc[64 L + 4 j + e]: lane 32 q + 16 L + 8 (e / 2) + lane / 4,
          // column 8 j + 2 (lane % 4) + e % 2 of the half
#pragma unroll
          for (int L = 0; L < 2; L++)
#pragma unroll
            for (int p4 = 0; p4 < 4; p4++) {
              uint32_t r[16];
              tmem_ld16x256b_x4_async(t0 + ((uint32_t)(16 * L) << 16) + (uint32_t)(32 * p4), r);
              tmem_wait16(r);
#pragma unroll
              for (int i = 0; i < 16; i++) acc[64 * L + 16 * p4 + i] += __uint_as_float(r[i]);
            }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            if constexpr (PAIR) mbar_arrive_cluster(leader_addr(&tempty[b]));  // the MMA issuer's barrier
            else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
          }
        }
      } else {
        for (int kb = kb0; kb < kb1; kb += a.kbd, c++) {
          const int b = c % NBUF;
          const uint32_t bph = (uint32_t)(c / NBUF) & 1u;
          if (!mbar_wait(&tfull[b], bph, a.err, ERR_ACCUM_WAIT, a.wait_cycles)) { ok = false; break; }
          tc_fence_after();
          const uint32_t t0 = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * BN + HC * h);
#pragma unroll
          for (int j = 0; j < HC; j += 16 * SCESS_TC_LDB) {
            uint32_t r[16 * SCESS_TC_LDB];
#pragma unroll
            for (int hh = 0; hh < SCESS_TC_LDB; hh++) tmem_ld16_async(t0 + (uint32_t)(j + 16 * hh), r + 16 * hh);
#pragma unroll
            for (int hh = 0; hh < SCESS_TC_LDB; hh++) tmem_wait16(r + 16 * hh);
#pragma unroll
            for (int i = 0; i < 16 * SCESS_TC_LDB; i++) acc[j + i] += __uint_as_float(r[i]);
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            if constexpr (PAIR) mbar_arrive_cluster(leader_addr(&tempty[b]));  // the MMA issuer's barrier
            else asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
          }
        }
      }
      asm volatile("bar.sync %0, 128;" ::"r"(bar) : "memory");  // colOff of this unit written
      if (!ok || errv) break;
      if (pc) {
        float *C = (float *)out.C;
        const float fa = s_falpha;
        const int cq = 2 * (lane & 3);
        // the warp's 32 row offsets, read back in the 16x256b row order
        rowOffS[h][row] = m < a.M ? rowOff : -1;
        __syncwarp();
        int64_t ro4[4];
#pragma unroll
        for (int s4 = 0; s4 < 4; s4++) ro4[s4] = rowOffS[h][32 * q + 8 * s4 + (lane >> 2)];
        // (two copies of the loop, stores and reductions: a choice per store
        // inside one loop costs the scheduling of the whole unrolled loop)
        if (!accum) {
#pragma unroll
          for (int j = 0; j < HC / 8; j++) {
            const int64_t co0 = colH[8 * j + cq], co1 = colH[8 * j + cq + 1];
#pragma unroll
            for (int s4 = 0; s4 < 4; s4++) {
              const int64_t ro = ro4[s4];
              const float v0 = fa * acc[64 * (s4 >> 1) + 4 * j + 2 * (s4 & 1)];
              const float v1 = fa * acc[64 * (s4 >> 1) + 4 * j + 2 * (s4 & 1) + 1];
              if (ro < 0) continue;
              float *d = C + ro + co0;
              if (co0 >= 0 && co1 == co0 + 1 && ((uintptr_t)d & 7) == 0) {
                *reinterpret_cast<float2 *>(d) = make_float2(v0, v1);
              } else {
                if (co0 >= 0) C[ro + co0] = v0;
                if (co1 >= 0) C[ro + co1] = v1;
              }
            }
          }
        } else {
          // Column quads: the lanes holding columns (c, c + 1) and (c + 2, c + 3)
          // of rows r and r + 8 swap half their values, so that the even lane adds
          // the quad of row r and the odd lane that of row r + 8, each with one
          // 16-byte reduction.
          const int odd = lane & 1;
          const int cq4 = 4 * ((lane >> 1) & 1);
#pragma unroll
          for (int j = 0; j < HC / 8; j++) {
            const int64_t co = colH[8 * j + cq4], co3 = colH[8 * j + cq4 + 3];
#pragma unroll
            for (int L = 0; L < 2; L++) {
              const int b = 64 * L + 4 * j;
              const float s0 = odd ? acc[b] : acc[b + 2], s1 = odd ? acc[b + 1] : acc[b + 3];
              const float r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
              const float r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
              const float v0 = fa * (odd ? r0 : acc[b]), v1 = fa * (odd ? r1 : acc[b + 1]);
              const float v2 = fa * (odd ? acc[b + 2] : r0), v3 = fa * (odd ? acc[b + 3] : r1);
              const int64_t ro = odd ? ro4[2 * L + 1] : ro4[2 * L];
              if (ro < 0 || co < 0) continue;
              float *d = C + ro + co;
              if (co3 == co + 3 && ((uintptr_t)d & 15) == 0) {
                red_add_v4(d, v0, v1, v2, v3);
              } else {  // (not expected: the host asks for quads only when aligned)
                const int64_t c1 = colH[8 * j + cq4 + 1], c2 = colH[8 * j + cq4 + 2];
                atomicAdd(C + ro + co, v0);
                if (c1 >= 0) atomicAdd(C + ro + c1, v1);
                if (c2 >= 0) atomicAdd(C + ro + c2, v2);
                if (co3 >= 0) atomicAdd(C + ro + co3, v3);
              }
            }
          }
        }
        __syncwarp();  // rowOffS read before the next unit rewrites it
        continue;
      }
      if (a.stcol[pg] && out.fp32 && out.beta == 0.0 && !a.partial) {  // (beta = 1: the generic path)
        // Tile staged through shared memory CH columns at a time, then each warp
        // stores its 32 rows with the lanes along the columns: for outputs whose
        // unit-stride index is a column index this writes contiguous runs.
        float *C = (float *)out.C;
        const float fa = s_falpha;
        constexpr int CH = SH::CH;
        rowOffS[h][row] = m < a.M ? rowOff : -1;
#pragma unroll
        for (int j0 = 0; j0 < HC; j0 += CH) {
          // each warp stages and stores only its own 32 rows: warp-level ordering
          __syncwarp();  // previous chunk read, rowOffS set
#pragma unroll
          for (int jj = 0; jj < CH; jj++) stage[h][jj][row] = fa * acc[j0 + jj];
          __syncwarp();
          if (BN == 256 && a.stvec[pg]) {  // (the (T) launch; einsums keep the scalar form)
            // every aligned quad of columns is a contiguous 16-byte run: lanes
            // take quad lane % QPR of row rr + lane / QPR (conflict-free reads:
            // the staging pitch is 2 mod 32 words)
            constexpr int QPR = CH / 4, RSTEP4 = 32 / QPR;
            const int cq = lane % QPR, rsub4 = lane / QPR;
            const int64_t co = colH[j0 + 4 * cq];
#pragma unroll
            for (int rr = 0; rr < 32; rr += RSTEP4) {
              const int r = 32 * q + rr + rsub4;
              const int64_t ro = rowOffS[h][r];
              if (ro >= 0 && co >= 0) {
                const float v0 = stage[h][4 * cq][r], v1 = stage[h][4 * cq + 1][r];
                const float v2 = stage[h][4 * cq + 2][r], v3 = stage[h][4 * cq + 3][r];
                float *d = C + ro + co;
                if (((uintptr_t)d & 15) == 0) {
                  *reinterpret_cast<float4 *>(d) = make_float4(v0, v1, v2, v3);
                } else {  // (not expected: the host asks for quads only when aligned)
                  d[0] = v0;
                  d[1] = v1;
                  d[2] = v2;
                  d[3] = v3;
                }
              }
            }
          } else {
            // lanes take column lane % CH of row rr + lane / CH (CH = 16: two rows a step)
            const int cl = lane % CH;
            const int rsub = lane / CH;
            constexpr int RSTEP = 32 / CH;
            const int64_t co = colH[j0 + cl];
#pragma unroll 4
            for (int rr = 0; rr < 32; rr += RSTEP) {
              const int r = 32 * q + rr + rsub;
              const int64_t ro = rowOffS[h][r];
              if (ro >= 0 && co >= 0) C[ro + co] = stage[h][cl][r];
            }
          }
        }
        continue;
      }
      if (m >= a.M) continue;
      if (a.partial) {
        const int sp = u / (tiles * nprob);
        float *P = a.partial + (int64_t)sp * a.part_stride;
#pragma unroll
        for (int j = 0; j < HC; j++) {
          const int n = n0 + j;
          if (n < a.N) P[(int64_t)m + (int64_t)a.M * n] = acc[j];
        }
        continue;
      }
      const double alpha = s_alpha;
      // beta == 1: fire-and-forget reductions (deterministic when each element
      // receives one per launch, as in every einsum launch; a (T) launch into
      // one W adds its three groups in whatever order they arrive); beta == 0:
      // plain stores; otherwise a batched read-modify-write.
      if (out.fp32) {
        float *C = (float *)out.C;
        const float fa = s_falpha, fb = (float)out.beta;
        if (out.beta == 1.0) {
#pragma unroll
          for (int j = 0; j < HC; j++) {
            const int64_t co = colH[j];
            if (co >= 0) atomicAdd(C + rowOff + co, fa * acc[j]);
          }
        } else if (out.beta == 0.0) {
#pragma unroll
          for (int j = 0; j < HC; j++) {
            const int64_t co = colH[j];
            if (co >= 0) C[rowOff + co] = fa * acc[j];
          }
        } else {
#pragma unroll
          for (int j = 0; j < HC; j += 16) {
            float old[16];
#pragma unroll
            for (int i = 0; i < 16; i++) {
              const int64_t co = colH[j + i];
              old[i] = co >= 0 ? C[rowOff + co] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < 16; i++) {
              const int64_t co = colH[j + i];
              if (co >= 0) C[rowOff + co] = fa * acc[j + i] + fb * old[i];
            }
          }
        }
      } else {
        double *C = (double *)out.C;
        const float fu = s_fuser;
        const long long sh = (long long)s_shift << 52;
        // alpha * acc as (double)(fu * acc) * 2^shift via the exponent field
        auto scaled = [&](float x) -> double {
          const float p = fu * x;
          return p == 0.0f ? 0.0 : __longlong_as_double(__double_as_longlong((double)p) + sh);
        };
        if (s_shift_ok && out.beta == 1.0) {
#pragma unroll
          for (int j = 0; j < HC; j++) {
            const int64_t co = colH[j];
            if (co >= 0) atomicAdd(C + rowOff + co, scaled(acc[j]));
          }
        } else if (s_shift_ok && out.beta == 0.0) {
#pragma unroll
          for (int j = 0; j < HC; j++) {
            const int64_t co = colH[j];
            if (co >= 0) C[rowOff + co] = scaled(acc[j]);
          }
        } else if (out.beta == 1.0) {
#pragma unroll
          for (int j = 0; j < HC; j++) {
            const int64_t co = colH[j];
            if (co >= 0) atomicAdd(C + rowOff + co, alpha * (double)acc[j]);
          }
        } else if (out.beta == 0.0) {
#pragma unroll
          for (int j = 0; j < HC; j++) {
            const int64_t co = colH[j];
            if (co >= 0) C[rowOff + co] = alpha * (double)acc[j];
          }
        } else {
#pragma unroll
          for (int j = 0; j < HC; j += 16) {
            double old[16];
#pragma unroll
            for (int i = 0; i < 16; i++) {
              const int64_t co = colH[j + i];
              old[i] = co >= 0 ? C[rowOff + co] : 0.0;
            }
#pragma unroll
            for (int i = 0; i < 16; i++) {
              const int64_t co = colH[j + i];
              if (co >= 0) C[rowOff + co] = alpha * (double)acc[j + i] + out.beta * old[i];
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  // pair: neither CTA leaves (or frees TMEM) while the other's copies, MMAs or
  // arrivals may still target it
  if constexpr (PAIR) cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    if constexpr (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                   "r"(SH::TMEM_COLS)
                   : "memory");
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                   "r"(SH::TMEM_COLS)
                   : "memory");
  }
}
#undef MMA_

__global__ void tc_reduce_kernel(TcOut out, int64_t M, int64_t N, int splits,
                                 const float *__restrict__ partial) {
  const int64_t MN = M * N;
  double alpha = out.alpha;
  if (out.scaleA) alpha /= *out.scaleA;
  if (out.scaleB) alpha /= *out.scaleB;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; z++) s += (double)partial[(int64_t)z * MN + e];
    const int64_t m = e % M, n = e / M;
    const int64_t off = out.baseC + out.rowC[m] + out.colC[n];
    if (out.fp32) {
      float *C = (float *)out.C;
      double val = alpha * s;
      if (out.beta != 0.0) val += out.beta * (double)C[off];
      C[off] = (float)val;
    } else {
      double *C = (double *)out.C;
      double val = alpha * s;
      if (out.beta != 0.0) val += out.beta * C[off];
      C[off] = val;
    }
  }
}

// max|x| over the gathered operand, as float bits (positive floats order like
// unsigned integers).
// max|x| over the gather of pack_split_kernel, in the same 32-row x 64-column
// tiles (offset tables staged in shared memory, eight independent loads a
// thread); a persistent grid walks the tiles.  The block's maximum goes to
// *maxbits as float bits with one atomicMax (exact: |x| rounded to FP32 is
// monotone in |x|).
// Row tiles of 32 rows along a group's smallest-stride label: row tile x holds
// rows r = pre + P (32 ft + t + E post), t < 32 (-1 past the label's extent),
// so that a tile's source values are contiguous when that stride is 1.
struct RowTiles {
  int64_t P = 1, E = 1, nft = 1, count = 0;
  static RowTiles make(int64_t rows, int64_t P, int64_t E) {
    RowTiles r;
    if (P < 1 || E < 1 || rows % (P * E) != 0) {  // not a product grouping: plain tiles
      P = 1;
      E = std::max<int64_t>(rows, 1);
    }
    r.P = P;
    r.E = E;
    r.nft = (E + 31) / 32;
    r.count = P * r.nft * (std::max<int64_t>(rows, 1) / (P * E));
    return r;
  }
  __device__ int64_t row(int64_t x, int t) const {
    const int64_t pre = x % P, rem = x / P, ft = rem % nft, post = rem / nft;
    const int64_t f = ft * 32 + t;
    return f < E ? pre + P * (f + E * post) : -1;
  }
};

// AFFINE: the offsets are r * rs and k * ks (no tables).
template <bool AFFINE>
__global__ void __launch_bounds__(256) maxabs_kernel(
    const double *__restrict__ src, const int64_t *__restrict__ rowOff, int64_t rows,
    const int64_t *__restrict__ kOff, int64_t K, int unitK, unsigned *__restrict__ maxbits,
    int64_t rs, int64_t ks, const RowTiles rt) {
  __shared__ int64_t sr[32], sk[64];
  __shared__ float red[8];
  const int t = threadIdx.x;
  const int64_t trow = rt.count, tk = (K + 63) / 64, ntiles = trow * tk;
  float m = 0.0f;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t k0 = (tile / trow) * 64;
    __syncthreads();  // previous tile's table reads done
    if (t < 32) {
      const int64_t r = rt.row(tile % trow, t);
      sr[t] = (r >= 0 && r < rows) ? (AFFINE ? r * rs : rowOff[r]) : -1;
    }
    else if (t < 96) sk[t - 32] = (k0 + t - 32 < K) ? (AFFINE ? (k0 + t - 32) * ks : kOff[k0 + t - 32]) : -1;
    __syncthreads();
    double x[8];
#pragma unroll
    for (int p = 0; p < 8; p++) {
      int rr, kk;
      if (unitK) { kk = t & 63; rr = (t >> 6) + 4 * p; }
      else { rr = t & 31; kk = (t >> 5) + 8 * p; }
      const int64_t ro = sr[rr], ko = sk[kk];
      x[p] = (ro >= 0 && ko >= 0) ? src[ro + ko] : 0.0;
    }
#pragma unroll
    for (int p = 0; p < 8; p++) m = fmaxf(m, fabsf((float)x[p]));
  }
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
  if ((t & 31) == 0) red[t >> 5] = m;
  __syncthreads();
  if (t == 0) {
    float b = 0.0f;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) b = fmaxf(b, red[q]);
    if (b > 0.0f) atomicMax(maxbits, __float_as_uint(b));
  }
}

// max|x| over n contiguous values (a gather that covers its source span).
__global__ void __launch_bounds__(256) maxabs_flat_kernel(const double *__restrict__ src, int64_t n,
                                                          unsigned *__restrict__ maxbits) {
  __shared__ float red[8];
  float m = 0.0f;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; e + 7 * stride < n; e += 8 * stride) {
    double x[8];
#pragma unroll
    for (int p = 0; p < 8; p++) x[p] = __ldg(src + e + p * stride);
#pragma unroll
    for (int p = 0; p < 8; p++) m = fmaxf(m, fabsf((float)x[p]));
  }
  for (; e < n; e += stride) m = fmaxf(m, fabsf((float)src[e]));
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.0f;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) b = fmaxf(b, red[q]);
    if (b > 0.0f) atomicMax(maxbits, __float_as_uint(b));
  }
}

// x s = hi + lo in FP16.  FP64 arithmetic runs at a small fraction of the FP32
// rate on GB300, so x is converted to FP32 once (relative error 2^-24, below
// the split's 2^-22) and the scaling (a power of two, exact) and the residual
// (exact: hi is xs rounded) are FP32 operations.  `fast` is false only for
// scales outside FP32's range (max|x| below ~2^-85), which keep the FP64 form.
struct HalfPair {
  __device__ static void split(double x, double s, float sf, bool fast, __half &hi, __half &lo) {
    if (fast) {
      const float xs = (float)x * sf;
      hi = __float2half_rn(xs);
      lo = __float2half_rn(xs - __half2float(hi));
    } else {
      const double xs = x * s;
      hi = __double2half(xs);
      lo = __double2half(xs - (double)__half2float(hi));
    }
  }
};

// Gathers rows x K FP64 values through offset tables into 16-bit hi/lo rows.
// FP16 format: values are scaled by s = 2^(15 - e), max|x| = f 2^e, f in [0.5, 1),
// which block (0,0) also stores for the epilogue.
// AFFINE: the offsets are r * rs and k * ks (no tables).
template <bool F16, bool AFFINE>
__global__ void __launch_bounds__(256) pack_split_kernel(
    const double *__restrict__ src, const int64_t *__restrict__ rowOff, int64_t rows,
    const int64_t *__restrict__ kOff, int64_t K, int unitK, uint16_t *__restrict__ dst,
    int64_t Kpad, const unsigned *__restrict__ maxbits, double *__restrict__ scale_out,
    int negate, int64_t rs, int64_t ks, const RowTiles rt) {
  __shared__ double tile[32][65];
  __shared__ int64_t sr[32], sk[64], srow[32];
  const int t = threadIdx.x;
  // row tiles on grid.x (up to 2^31 - 1), K blocks on grid.y (<= 65535)
  const int64_t k0 = (int64_t)blockIdx.y * 64;
  if (t < 32) {
    const int64_t r = rt.row(blockIdx.x, t);
    srow[t] = (r >= 0 && r < rows) ? r : -1;
    sr[t] = srow[t] >= 0 ? (AFFINE ? r * rs : rowOff[r]) : -1;
  }
  else if (t < 96) sk[t - 32] = (k0 + t - 32 < K) ? (AFFINE ? (k0 + t - 32) * ks : kOff[k0 + t - 32]) : -1;
  double s = 1.0;
  if (F16) {
    const float mx = __uint_as_float(*maxbits);
    if (mx > 0.0f) {
      int e;
      frexpf(mx, &e);
      s = ldexp(1.0, 15 - e);
    }
    if (blockIdx.x == 0 && blockIdx.y == 0 && t == 0) *scale_out = s;
  }
  const bool fast = s <= 0x1p100 && s >= 0x1p-100;
  const float sf = fast ? (float)s : 1.0f;
  __syncthreads();
#pragma unroll
  for (int p = 0; p < 8; p++) {
    int rr, kk;
    if (unitK) { kk = t & 63; rr = (t >> 6) + 4 * p; }
    else { rr = t & 31; kk = (t >> 5) + 8 * p; }
    const int64_t ro = sr[rr], ko = sk[kk];
    // negation as a sign-bit flip (exact, no FP64 arithmetic)
    tile[rr][kk] = (ro >= 0 && ko >= 0)
                       ? __longlong_as_double(__double_as_longlong(src[ro + ko]) ^
                                              ((long long)negate << 63))
                       : 0.0;
  }
  __syncthreads();
  const int rr = t >> 3, ch = t & 7;
  __align__(16) uint16_t hi[8];
  __align__(16) uint16_t lo[8];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const double x = tile[rr][ch * 8 + j];
    if (F16) {
      __half h, l;
      HalfPair::split(x, s, sf, fast, h, l);
      hi[j] = __half_as_ushort(h);
      lo[j] = __half_as_ushort(l);
    } else {
      // BF16 shares FP32's exponent range: split the FP32 value (see HalfPair)
      const float xf = (float)x;
      const __nv_bfloat16 h = __float2bfloat16_rn(xf);
      hi[j] = __bfloat16_as_ushort(h);
      lo[j] = __bfloat16_as_ushort(__float2bfloat16_rn(xf - __bfloat162float(h)));
    }
  }
  const int64_t r = srow[rr];
  if (r < 0) return;  // past the label's extent (padding rows are cleared by the host)
  if (k0 + ch * 8 >= Kpad) return;  // Kpad a multiple of 32: the tile's last 32 columns are past it
  const int64_t base = r * 2 * Kpad + k0 + ch * 8;
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

// Boxes of box_rows x bk 16-bit values: bk = 64 (128-byte rows, SWIZZLE_128B)
// or 32 (64-byte rows, SWIZZLE_64B), matching the kernel's K block.
CUtensorMap make_map(const void *base, int64_t rows_pad, int64_t Kpad, int box_rows, int bk,
                     TcFormat fmt) {
  if (bk != 64 && bk != 32) throw Error(SCESS_ERR_INVALID, "tc_gemm: K block of a map");
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  cuuint64_t dims[2] = {(cuuint64_t)(2 * Kpad), (cuuint64_t)rows_pad};
  cuuint64_t strides[1] = {(cuuint64_t)(2 * Kpad * 2)};
  cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = get_encode()(&m, fmt == TcFormat::FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                      : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                            2, const_cast<void *>(base), dims, strides,
                            box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(SCESS_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return m;
}

}  // namespace

int TcEngine::tile_n(int64_t) { return V2_BN; }

CUtensorMap TcEngine::map_of(const Packed &p, int box_rows, int bk) {
  return make_map(p.p(), p.rows_pad, p.Kpad, box_rows, bk, p.fmt);
}

// K block of the kernels: 64 (128-byte rows, SWIZZLE_128B).  (A 256-wide
// kernel with 32-wide blocks in 4 stages measured 5 % slower.)
int TcEngine::k_block(int) { return 64; }

namespace {

// One-time kernel attributes and capabilities of this device: the 256-wide
// kernels' register count (their setmaxnreg split assumes kLaunchRegs256) and
// how many cluster pairs of the pair kernel are co-resident.
struct KernelSetup {
  bool wide_ok = false, pair_ok = false;
  int pair_clusters = 0;
};
const KernelSetup &kernel_setup() {
  static KernelSetup k;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(tc_gemm_kernel<128, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)TcShape<128, 64>::SMEM_BYTES);
    cudaFuncSetAttribute(tc_gemm_kernel<256, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)TcShape<256, 64>::SMEM_BYTES);
    // The 256-wide kernels' setmaxnreg split assumes they are launched with
    // exactly kLaunchRegs256 registers a thread (3 x 168 = 56 + 2 x 224 per scheduler).
    cudaFuncAttributes fa, fc;
    k.wide_ok = cudaFuncGetAttributes(&fa, tc_gemm_kernel<256, 64>) == cudaSuccess &&
              fa.numRegs == kLaunchRegs256;
    using SP = TcShape<256, 64, true>;
    if (cudaFuncSetAttribute(tc_gemm_kernel<256, 64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)SP::SMEM_BYTES) == cudaSuccess &&
        cudaFuncGetAttributes(&fc, tc_gemm_kernel<256, 64, true>) == cudaSuccess &&
        fc.numRegs == kLaunchRegs256) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 2;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(2 * (kNumSMs / 2));
      cfg.blockDim = dim3(SP::THREADS);
      cfg.dynamicSmemBytes = SP::SMEM_BYTES;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, tc_gemm_kernel<256, 64, true>, &cfg) == cudaSuccess && n > 0) {
        k.pair_clusters = n;
        k.pair_ok = true;
      }
    }
    cudaGetLastError();
  });
  return k;
}

}  // namespace

bool TcEngine::pair_available() { return kernel_setup().pair_ok; }

void tc_gemm_launch_grouped(const TcProblemSet &ps, TcFormat fmt, const TcOut &out, int nseg,
                            int splits, float *partial, unsigned *err, cudaStream_t stream,
                            const TcWaitDiag &diag) {
  const KernelSetup &ks = kernel_setup();
  const bool wide_ok = ks.wide_ok, pair_ok = ks.pair_ok;
  const int pair_clusters = ks.pair_clusters;
  const int bn = ps.bn == 256 ? 256 : 128;
  if (bn == 256 && !wide_ok) throw Error(SCESS_ERR_UNSUPPORTED, "tc_gemm: 256-wide kernel unavailable");
  // the maps' boxes were made for this K block (a mismatch would overrun the stages)
  const int bk = TcEngine::k_block(bn);
  if (ps.bk != bk) throw Error(SCESS_ERR_INVALID, "tc_gemm: maps built for another K block");
  const bool pair = ps.pair;
  if (pair && (bn != 256 || bk != 64)) throw Error(SCESS_ERR_INVALID, "tc_gemm: pair needs the 256 x 64 kernel");
  if (pair && !pair_ok) throw Error(SCESS_ERR_UNSUPPORTED, "tc_gemm: cluster-pair kernel unavailable");
  const int bm = pair ? 2 * TC_BM : TC_BM;  // rows of a work unit
  if (ps.M <= 0 || ps.N <= 0 || ps.ny <= 0 || ps.nz <= 0 || ps.ng <= 0) return;
  if (ps.ng > 3) throw Error(SCESS_ERR_INVALID, "tc_gemm: groups");
  if (nseg != 1 && nseg != 3) throw Error(SCESS_ERR_INVALID, "tc_gemm: nseg");
  if (ps.nseg < 1 || ps.nseg > 4) throw Error(SCESS_ERR_INVALID, "tc_gemm: segments");
  if (ps.M > INT32_MAX || ps.N > INT32_MAX) throw Error(SCESS_ERR_INVALID, "tc_gemm: dimension too large");
  TcArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = (int)ps.M;
  a.N = (int)ps.N;
  a.tiles_m = (int)ceil_div(ps.M, bm);
  a.tiles_n = (int)ceil_div(ps.N, bn);
  a.ny = ps.ny;
  a.nz = ps.nz;
  a.ng = ps.ng;
  a.nseg = ps.nseg;
  int kbt = 0;
  for (int s = 0; s < ps.nseg; s++) {
    const TcSegment &g = ps.seg[s];
    // a segment may use 32-wide K blocks in the 64-wide kernel (maps with
    // 32-wide boxes, K padded to 32); otherwise the kernel's K block
    const int sbk = g.bk ? g.bk : bk;
    if (!(sbk == bk || (sbk == 32 && bk == 64)))
      throw Error(SCESS_ERR_INVALID, "tc_gemm: segment K block");
    if (g.Kpad % sbk != 0 || g.Kpad <= 0 || 2 * g.Kpad > INT32_MAX)
      throw Error(SCESS_ERR_INVALID, "tc_gemm: segment K not a multiple of its K block");
    for (int q = 0; q < ps.ng; q++) {
      const int64_t maxA = g.rowA0[q] + (int64_t)(ps.ny - 1) * g.rowAy[q] +
                           (int64_t)(ps.nz - 1) * g.rowAz[q] + a.tiles_m * bm;
      const int64_t maxB = g.rowB0[q] + (int64_t)(ps.ny - 1) * g.rowBy[q] +
                           (int64_t)(ps.nz - 1) * g.rowBz[q] + a.tiles_n * bn;
      if (maxA > INT32_MAX || maxB > INT32_MAX || g.rowA0[q] < 0 || g.rowB0[q] < 0 ||
          g.rowAy[q] < 0 || g.rowAz[q] < 0 || g.rowBy[q] < 0 || g.rowBz[q] < 0)
        throw Error(SCESS_ERR_INVALID, "tc_gemm: row coordinates");
    }
    a.seg[s].mapA = g.mapA;
    a.seg[s].mapB = g.mapB;
    a.seg[s].nkb = (int)(g.Kpad / sbk);
    a.seg[s].bk = sbk;
    a.seg[s].kpad = (int)g.Kpad;
    a.seg[s].negA = g.negate ? 1 : 0;
    for (int q = 0; q < 3; q++) {
      a.seg[s].rowA0[q] = g.rowA0[q];
      a.seg[s].rowAy[q] = g.rowAy[q];
      a.seg[s].rowAz[q] = g.rowAz[q];
      a.seg[s].rowB0[q] = g.rowB0[q];
      a.seg[s].rowBy[q] = g.rowBy[q];
      a.seg[s].rowBz[q] = g.rowBz[q];
    }
    kbt += a.seg[s].nkb;
  }
  a.kb_total = kbt;
  if (splits < 1) splits = 1;
  if (ps.ny * ps.nz * ps.ng > 1) splits = 1;
  if (splits > kbt) splits = kbt;
  const int kbs = (int)ceil_div(kbt, splits);
  splits = (int)ceil_div(kbt, kbs);
  a.kb_per_split = kbs;
  a.splits = splits;
  a.f16 = fmt == TcFormat::FP16 ? 1 : 0;
  a.split3 = nseg == 3 ? 1 : 0;
  a.kbd = (ps.kbd == 2 || ps.kbd == 4) ? ps.kbd : 1;
  for (int q = 0; q < 3; q++) {
    a.cy[q] = ps.cy[q];
    a.cz[q] = ps.cz[q];
    a.cg[q] = ps.cg[q];
    a.rowCg[q] = ps.rowC[q];
    a.colCg[q] = ps.colC[q];
    a.stcol[q] = ps.store_by_column[q] ? 1 : 0;
    a.stvec[q] = ps.store_by_column[q] && ps.store_quads[q] ? 1 : 0;
  }
  a.partial = splits > 1 ? partial : nullptr;
  a.part_stride = ps.M * ps.N;
  a.err = err;
  a.wait_cycles = diag.wait_cycles;
  a.withhold_first = diag.withhold_first ? 1 : 0;
  if (splits > 1 && !partial) throw Error(SCESS_ERR_INVALID, "tc_gemm: split-K needs partials");
  TcMaps maps;
  for (int i = 0; i < 6; i++) maps.m[i] = ps.maps[std::min(i, ps.nmaps - 1)];
  {  // problems per group: all ny nz, or the ny (ny + 1) / 2 with y >= z
    int64_t start = 0;
    for (int g = 0; g < ps.ng; g++) {
      a.tri[g] = ps.tri[g] ? 1 : 0;
      if (a.tri[g] && (ps.ny != ps.nz || bn != 256))
        throw Error(SCESS_ERR_INVALID, "tc_gemm: triangular groups need ny == nz and the 256-wide kernel");
      a.gstart[g] = (int)start;
      start += a.tri[g] ? (int64_t)ps.ny * (ps.ny + 1) / 2 : (int64_t)ps.ny * ps.nz;
    }
    if (start > INT32_MAX) throw Error(SCESS_ERR_INVALID, "tc_gemm: too many problems");
    a.gstart[ps.ng] = (int)start;
  }
  const int64_t units = (int64_t)a.tiles_m * a.tiles_n * a.gstart[ps.ng] * splits;
  if (units > INT32_MAX) throw Error(SCESS_ERR_INVALID, "tc_gemm: too many work units");
  const unsigned grid = (unsigned)std::min<int64_t>(units, kNumSMs);
  if (pair) {
    // one persistent pair per co-resident cluster slot
    using SP = TcShape<256, 64, true>;
    const int64_t ncl = std::min<int64_t>(units, pair_clusters);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = dim3((unsigned)(2 * ncl));
    cfg.blockDim = dim3(SP::THREADS);
    cfg.dynamicSmemBytes = SP::SMEM_BYTES;
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = ps.pdl ? 2 : 1;
    SCESS_CUDA(cudaLaunchKernelEx(&cfg, tc_gemm_kernel<256, 64, true>, maps, out, a));
  } else if (bn == 256)
    tc_gemm_kernel<256, 64><<<grid, TcShape<256, 64>::THREADS, TcShape<256, 64>::SMEM_BYTES, stream>>>(
        maps, out, a);
  else
    tc_gemm_kernel<128, 64><<<grid, TcShape<128, 64>::THREADS, TcShape<128, 64>::SMEM_BYTES, stream>>>(
        maps, out, a);
  SCESS_CHECK_LAUNCH();
  if (splits > 1) {
    const int64_t MN = ps.M * ps.N;
    tc_reduce_kernel<<<(unsigned)std::min<int64_t>(ceil_div(MN, 256), 8192), 256, 0, stream>>>(
        out, ps.M, ps.N, splits, partial);
    SCESS_CHECK_LAUNCH();
  }
}

void tc_gemm_launch_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t rowA0,
                         int64_t M, int64_t rowB0, int64_t N, int bn, TcFormat fmt,
                         const TcOut &out, int nseg, int splits, float *partial, unsigned *err,
                         cudaStream_t stream, const TcWaitDiag &diag) {
  (void)bn;
  TcProblemSet ps;
  ps.maps[0] = ma;
  ps.maps[1] = mb;
  ps.nmaps = 2;
  ps.M = M;
  ps.N = N;
  ps.nseg = 1;
  ps.seg[0].mapA = 0;
  ps.seg[0].mapB = 1;
  ps.seg[0].Kpad = Kpad;
  ps.seg[0].rowA0[0] = rowA0;
  ps.seg[0].rowB0[0] = rowB0;
  tc_gemm_launch_grouped(ps, fmt, out, nseg, splits, partial, err, stream, diag);
}

void TcEngine::gemm_maps(const CUtensorMap &ma, const CUtensorMap &mb, int64_t Kpad, int64_t Kreal,
                         int64_t rowA0, int64_t M, int64_t rowB0, int64_t N, const TcOut &out,
                         int nseg, cudaStream_t stream) {
  TimedScope ts(ctx_.timer, "tc_gemm", 2.0 * M * N * Kreal, 0.0, stream ? stream : ctx_.stream);
  tc_gemm_launch_maps(ma, mb, Kpad, rowA0, M, rowB0, N, tile_n(N), fmt_, out, nseg, 1, nullptr,
                      err_.as<unsigned>(), stream ? stream : ctx_.stream, take_diag());
}

TcWaitDiag TcEngine::take_diag() {
  TcWaitDiag d = diag_;
  diag_ = TcWaitDiag();  // one launch only
  return d;
}

// ---------------------------------------------------------------------------------------------

TcEngine::TcEngine(Ctx &ctx) : ctx_(ctx) {
  // operands in the scaled FP16 split (the unscaled BF16 split is 32x coarser)
  fmt_ = TcFormat::FP16;
  err_.alloc(sizeof(unsigned) * 4);
  SCESS_CUDA(cudaMemsetAsync(err_.as<void>(), 0, sizeof(unsigned) * 4, ctx_.stream));
}

TcEngine::~TcEngine() = default;

void TcEngine::gemm_grouped(const TcProblemSet &ps, const TcOut &out, double flops,
                            const char *name, cudaStream_t stream) {
  TimedScope ts(ctx_.timer, name, flops, 0.0, stream ? stream : ctx_.stream);
  tc_gemm_launch_grouped(ps, fmt_, out, 3, 1, nullptr, err_.as<unsigned>(),
                         stream ? stream : ctx_.stream, take_diag());
}

// GB300's FP64 units run the table GEMM at ~1 TFLOP/s for large tiles and at a
// fraction of that when M or N is small (a 64x64 tile holding a 20x20 result),
// so any contraction above ~2e7 FLOPs is faster on the tensor cores, even with
// most of a 128x128 tile idle; matrix-vector shapes stay on the FP64 GEMV.
bool TcEngine::worth_it(const EinsumPlan &pl) {
  const int64_t mn = std::min(pl.M, pl.N);
  return mn >= 4 && pl.K >= 16 && 2.0 * pl.M * pl.N * pl.K >= 2.0e7;
}

namespace {
// Persistent grid of maxabs_kernel: at most 8 blocks an SM, at least one tile each.
unsigned maxabs_blocks(const RowTiles &rt, int64_t K) {
  const int64_t tiles = rt.count * ceil_div(std::max<int64_t>(K, 1), 64);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(tiles, 8 * kNumSMs));
}

// Rows [rows, rows_pad) of a packed operand are zero.
void clear_pad_rows(uint16_t *dst, int64_t rows, int64_t rows_pad, int64_t Kpad, cudaStream_t s) {
  if (rows_pad > rows)
    SCESS_CUDA(cudaMemsetAsync(dst + rows * 2 * Kpad, 0,
                               (size_t)(rows_pad - rows) * 2 * Kpad * sizeof(uint16_t), s));
}
}  // namespace

void TcEngine::pack(const double *src, const int64_t *rowOff, int64_t rows, const int64_t *kOff,
                    int64_t K, bool unitK, int64_t row_align, Packed &out, int64_t rs,
                    int64_t ks, int64_t rP, int64_t rE, bool dense) {
  const bool aff = rs >= 0 && ks >= 0;
  const RowTiles rt = RowTiles::make(rows, rP, rE > 0 ? rE : rows);
  const int64_t Kpad = round_up(std::max<int64_t>(K, 1), TC_BK);
  const int64_t rows_pad = round_up(std::max<int64_t>(rows, 1), std::max<int64_t>(row_align, 32));
  const size_t bytes = (size_t)rows_pad * 2 * Kpad * sizeof(uint16_t);
  if (out.mem.bytes() < bytes || !out.aux.bytes()) {
    ctx_.sync();
    if (out.mem.bytes() < bytes) out.mem.alloc(bytes);
    if (!out.aux.bytes()) out.aux.alloc(16);
  }
  out.rows = rows;
  out.rows_pad = rows_pad;
  out.K = K;
  out.Kpad = Kpad;
  out.fmt = fmt_;
  // timed per contraction: "pack[spec]" inside an einsum ("tc_gemm[spec]")
  const std::string tname =
      timer_name_ && std::strncmp(timer_name_, "tc_gemm", 7) == 0 ? std::string("pack") + (timer_name_ + 7)
                                                                  : std::string("pack_split");
  TimedScope ts(ctx_.timer, tname.c_str(), 0.0,
                (double)rows * K * 8 + (double)rows_pad * Kpad * 4, ctx_.stream);
  unsigned *maxbits = out.aux.as<unsigned>();
  double *scale = reinterpret_cast<double *>(out.aux.as<char>() + 8);
  if (Kpad / 64 > 65535 || rt.count > INT32_MAX) throw Error(SCESS_ERR_INVALID, "pack: too large");
  dim3 grid((unsigned)rt.count, (unsigned)(Kpad / 64));
  uint16_t *dst = out.mem.as<uint16_t>();
  clear_pad_rows(dst, rows, rows_pad, Kpad, ctx_.stream);
  const int u = unitK ? 1 : 0;
  const unsigned *hint = nullptr;
  for (const MaxHint &h : hints_)
    if (h.p == src) hint = hint_words_.as<unsigned>() + h.slot;
  if (fmt_ == TcFormat::FP16 && hint) {  // the tensor's maximum, reduced once
    if (aff)
      pack_split_kernel<true, true><<<grid, 256, 0, ctx_.stream>>>(src, nullptr, rows, nullptr, K, u, dst,
                                                                   Kpad, hint, scale, 0, rs, ks, rt);
    else
      pack_split_kernel<true, false><<<grid, 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K, u, dst,
                                                                    Kpad, hint, scale, 0, 0, 0, rt);
  } else if (fmt_ == TcFormat::FP16) {
    SCESS_CUDA(cudaMemsetAsync(maxbits, 0, sizeof(unsigned), ctx_.stream));
    const int64_t n = rows * K;
    if (dense || (aff && ((rs == 1 && ks == rows) || (ks == 1 && rs == K)))) {  // the gather is src[0, n)
      const unsigned blocks =
          (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256 * 8), 8 * kNumSMs));
      maxabs_flat_kernel<<<blocks, 256, 0, ctx_.stream>>>(src, n, maxbits);
    } else if (aff) {
      maxabs_kernel<true><<<maxabs_blocks(rt, K), 256, 0, ctx_.stream>>>(src, nullptr, rows, nullptr,
                                                                        K, u, maxbits, rs, ks, rt);
    } else {
      maxabs_kernel<false><<<maxabs_blocks(rt, K), 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K,
                                                                         u, maxbits, 0, 0, rt);
    }
    SCESS_CHECK_LAUNCH();
    if (aff)
      pack_split_kernel<true, true><<<grid, 256, 0, ctx_.stream>>>(src, nullptr, rows, nullptr, K, u, dst,
                                                                   Kpad, maxbits, scale, 0, rs, ks, rt);
    else
      pack_split_kernel<true, false><<<grid, 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K, u, dst,
                                                                    Kpad, maxbits, scale, 0, 0, 0, rt);
  } else {
    const double one = 1.0;
    SCESS_CUDA(cudaMemcpyAsync(scale, &one, sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
    if (aff)
      pack_split_kernel<false, true><<<grid, 256, 0, ctx_.stream>>>(src, nullptr, rows, nullptr, K, u, dst,
                                                                    Kpad, maxbits, scale, 0, rs, ks, rt);
    else
      pack_split_kernel<false, false><<<grid, 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K, u, dst,
                                                                     Kpad, maxbits, scale, 0, 0, 0, rt);
  }
  SCESS_CHECK_LAUNCH();
}

void TcEngine::add_max_hint(const double *p, int64_t n) {
  constexpr int kSlots = 8;
  if (fmt_ != TcFormat::FP16 || !p || n <= 0 || (int)hints_.size() >= kSlots) return;
  if (!hint_words_.bytes()) {
    ctx_.sync();
    hint_words_.alloc(kSlots * sizeof(unsigned));
  }
  const int slot = (int)hints_.size();
  unsigned *word = hint_words_.as<unsigned>() + slot;
  TimedScope ts(ctx_.timer, "pack_max", 0.0, (double)n * 8, ctx_.stream);
  SCESS_CUDA(cudaMemsetAsync(word, 0, sizeof(unsigned), ctx_.stream));
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256 * 8), 8 * kNumSMs));
  maxabs_flat_kernel<<<blocks, 256, 0, ctx_.stream>>>(p, n, word);
  SCESS_CHECK_LAUNCH();
  hints_.push_back({p, slot});
}

void TcEngine::clear_max_hints() {
  hints_.clear();
  reuse_.clear();
}

void TcEngine::maxabs_into(const double *src, const int64_t *rowOff, int64_t rows,
                           const int64_t *kOff, int64_t K, bool unitK, unsigned *maxbits) {
  if (rows <= 0 || K <= 0) return;
  const RowTiles rt = RowTiles::make(rows, 1, rows);
  maxabs_kernel<false><<<maxabs_blocks(rt, K), 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K,
                                                                     unitK ? 1 : 0, maxbits, 0, 0, rt);
  SCESS_CHECK_LAUNCH();
}

void TcEngine::pack_with_max(const double *src, const int64_t *rowOff, int64_t rows,
                             const int64_t *kOff, int64_t K, bool unitK, int64_t row_align,
                             const unsigned *maxbits, bool negate, Packed &out, int64_t k_align) {
  if (k_align != 32 && k_align != 64) throw Error(SCESS_ERR_INVALID, "pack: K alignment");
  const int64_t Kpad = round_up(std::max<int64_t>(K, 1), k_align);
  const int64_t rows_pad = round_up(std::max<int64_t>(rows, 1), std::max<int64_t>(row_align, 32));
  const size_t bytes = (size_t)rows_pad * 2 * Kpad * sizeof(uint16_t);
  if (out.mem.bytes() < bytes || !out.aux.bytes()) {
    ctx_.sync();
    if (out.mem.bytes() < bytes) out.mem.alloc(bytes);
    if (!out.aux.bytes()) out.aux.alloc(16);
  }
  out.rows = rows;
  out.rows_pad = rows_pad;
  out.K = K;
  out.Kpad = Kpad;
  out.fmt = fmt_;
  TimedScope ts(ctx_.timer, "pack_split", 0.0,
                (double)rows * K * 8 + (double)rows_pad * Kpad * 4, ctx_.stream);
  double *scale = reinterpret_cast<double *>(out.aux.as<char>() + 8);
  const RowTiles rt = RowTiles::make(rows, 1, rows);
  if (ceil_div(Kpad, 64) > 65535 || rt.count > INT32_MAX) throw Error(SCESS_ERR_INVALID, "pack: too large");
  dim3 grid((unsigned)rt.count, (unsigned)ceil_div(Kpad, 64));
  clear_pad_rows(out.mem.as<uint16_t>(), rows, rows_pad, Kpad, ctx_.stream);
  if (fmt_ == TcFormat::FP16) {
    pack_split_kernel<true, false><<<grid, 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K, unitK ? 1 : 0,
                                                                  out.mem.as<uint16_t>(), Kpad, maxbits,
                                                                  scale, negate ? 1 : 0, 0, 0, rt);
  } else {
    const double one = 1.0;
    SCESS_CUDA(cudaMemcpyAsync(scale, &one, sizeof(double), cudaMemcpyHostToDevice, ctx_.stream));
    pack_split_kernel<false, false><<<grid, 256, 0, ctx_.stream>>>(src, rowOff, rows, kOff, K, unitK ? 1 : 0,
                                                                   out.mem.as<uint16_t>(), Kpad, maxbits,
                                                                   scale, negate ? 1 : 0, 0, 0, rt);
  }
  SCESS_CHECK_LAUNCH();
}

void TcEngine::gemm(const Packed &A, int64_t rowA0, int64_t M, const Packed &B, int64_t rowB0,
                    int64_t N, const TcOut &out, int nseg, int force_splits) {
  if (A.Kpad != B.Kpad) throw Error(SCESS_ERR_INVALID, "tc gemm: K mismatch");
  const int nkb = (int)(A.Kpad / TC_BK);
  int splits = force_splits;
  if (splits <= 0) {
    const int64_t tiles = ceil_div(M, TC_BM) * ceil_div(N, V2_BN);
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
  TimedScope ts(ctx_.timer, timer_name_ ? timer_name_ : "tc_gemm", 2.0 * M * N * A.K, 0.0,
                ctx_.stream);
  TcOut o = out;
  set_scales(o, A, B);
  const int bn = tile_n(N);
  const CUtensorMap ma = map_of(A, TC_BM), mb = map_of(B, bn);
  tc_gemm_launch_maps(ma, mb, A.Kpad, rowA0, M, rowB0, N, bn, fmt_, o, nseg, splits, partial,
                      err_.as<unsigned>(), ctx_.stream, take_diag());
}

void TcEngine::clear_cache(const void *owner) {
  for (auto it = cache_.begin(); it != cache_.end();) {
    if (it->second.first == owner) it = cache_.erase(it);
    else ++it;
  }
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

void TcEngine::table_gemm(const TableGemm &g, const char *name) {
  const std::string tname = std::string("tc_gemm[") + name + "]";
  timer_name_ = tname.c_str();
  pack(g.A + g.baseA, g.rowA, g.M, g.kA, g.K, false, TC_BM, tmpA_);
  pack(g.B + g.baseB, g.colB, g.N, g.kB, g.K, false, TC_BM, tmpB_);
  TcOut o;
  o.C = g.C + g.baseC;
  o.fp32 = 0;
  o.rowC = g.rowC;
  o.colC = g.colC;
  o.alpha = g.alpha;
  o.beta = g.beta;
  gemm(tmpA_, 0, g.M, tmpB_, 0, g.N, o, 3);
  timer_name_ = nullptr;
}

void TcEngine::contract(const EinsumPlan &pl, double alpha, const double *A, const double *B,
                        double beta, double *C, bool constA, bool constB) {
  // Epilogue lanes walk the GEMM rows: put C's unit-stride index there.
  const bool swap = pl.cUnitM ? false : (pl.cUnitN ? true : (pl.M < 64 && pl.N >= 64));
  const int64_t *rowX = swap ? pl.d_colB : pl.d_rowA, *kX = swap ? pl.d_kB : pl.d_kA;
  const int64_t *rowY = swap ? pl.d_rowA : pl.d_colB, *kY = swap ? pl.d_kA : pl.d_kB;
  const double *X = swap ? B : A, *Y = swap ? A : B;
  const bool cX = swap ? constB : constA, cY = swap ? constA : constB;
  const bool uX = swap ? pl.bUnitK : pl.aUnitK, uY = swap ? pl.aUnitK : pl.bUnitK;
  const int64_t MX = swap ? pl.N : pl.M, NY = swap ? pl.M : pl.N;

  struct Hint {
    int64_t rs, ks, P, E;
    bool dense;
  };
  const Hint hA{pl.aRowStride, pl.aKStride, pl.aRowP, pl.aRowE, pl.aDense};
  const Hint hB{pl.bColStride, pl.bKStride, pl.bColP, pl.bColE, pl.bDense};
  const Hint &hX = swap ? hB : hA, &hY = swap ? hA : hB;
  auto table_hash = [](const std::vector<int64_t> &r, const std::vector<int64_t> &k) {
    uint64_t x = 1469598103934665603ull;  // FNV-1a over sizes and entries
    auto mix = [&](uint64_t v) {
      for (int b = 0; b < 8; b++) {
        x ^= (v >> (8 * b)) & 0xffu;
        x *= 1099511628211ull;
      }
    };
    mix(r.size());
    for (int64_t e : r) mix((uint64_t)e);
    mix(k.size());
    for (int64_t e : k) mix((uint64_t)e);
    return x | 1ull;  // (0 = not yet computed)
  };
  auto get = [&](const double *src, const int64_t *rows, int64_t nrows, const int64_t *ks,
                 bool unitK, bool isConst, const char *tag, Packed &tmp,
                 const Hint &h) -> const Packed & {
    if (!isConst) {
      bool hinted = false;
      for (const MaxHint &mh : hints_) hinted = hinted || mh.p == src;
      if (!hinted) {
        pack(src, rows, nrows, ks, pl.K, unitK, TC_BM, tmp, h.rs, h.ks, h.P, h.E, h.dense);
        return tmp;
      }
      const bool isA = rows == pl.d_rowA;
      uint64_t &hs = isA ? pl.hashA : pl.hashB;
      if (!hs) hs = isA ? table_hash(pl.rowA, pl.kA) : table_hash(pl.colB, pl.kB);
      const std::string key = std::to_string((uintptr_t)src) + "|" + std::to_string(hs) + "|" +
                              std::to_string(nrows) + "|" + std::to_string(pl.K) + (unitK ? "u" : "s");
      auto it = reuse_.find(key);
      if (it != reuse_.end()) return *it->second;
      auto pk = std::make_unique<Packed>();
      pack(src, rows, nrows, ks, pl.K, unitK, TC_BM, *pk, h.rs, h.ks, h.P, h.E, h.dense);
      auto &ref = *pk;
      reuse_[key] = std::move(pk);
      return ref;
    }
    std::string key = pl.key + tag + std::to_string((uintptr_t)src);
    auto it = cache_.find(key);
    if (it != cache_.end() && it->second.first == owner_) return *it->second.second;
    auto pk = std::make_unique<Packed>();
    pack(src, rows, nrows, ks, pl.K, unitK, TC_BM, *pk, h.rs, h.ks, h.P, h.E, h.dense);
    auto &ref = *pk;
    cache_[key] = std::make_pair(owner_, std::move(pk));
    return ref;
  };
  const std::string tname = "tc_gemm[" + pl.spec + "]";
  timer_name_ = tname.c_str();
  const Packed &PX = get(X, rowX, MX, kX, uX, cX, swap ? "#B" : "#A", tmpA_, hX);
  const Packed &PY = get(Y, rowY, NY, kY, uY, cY, swap ? "#A" : "#B", tmpB_, hY);
  TcOut o;
  o.C = C;
  o.fp32 = 0;
  o.rowC = swap ? pl.d_colC : pl.d_rowC;
  o.colC = swap ? pl.d_rowC : pl.d_colC;
  o.alpha = alpha;
  o.beta = beta;
  gemm(PX, 0, MX, PY, 0, NY, o, 3);
  timer_name_ = nullptr;
}

}  // namespace scess
