// FP64 contraction engine and bandwidth-bound kernels of the closed-shell CC path.
//
// GB300 runs FP64 at a small fraction of its tensor rate, so the FP64 GEMM is
// DFMA-bound at any reasonable tile size: one 64x64 tile per 256-thread CTA with
// 4x4 register blocking, operands gathered through offset tables (the einsum
// permutation is fused into the tile loads), deterministic split-K when the
// output has too few tiles to cover the 152 SMs.
#include "common.cuh"
#include "kernels.h"

namespace scess {

namespace {

constexpr int BM = 64, BN = 64, BK = 16;

__global__ void __launch_bounds__(256) dgemm_table_kernel(TableGemm g, int64_t kChunk,
                                                          double *partial) {
  __shared__ double As[BK][BM];
  __shared__ double Bs[BK][BN];
  __shared__ int64_t sRowA[BM], sColB[BN], sKA[BK], sKB[BK];
  const int t = threadIdx.x;
  const int64_t m0 = (int64_t)blockIdx.x * BM, n0 = (int64_t)blockIdx.y * BN;
  const int64_t kb = (int64_t)blockIdx.z * kChunk;
  const int64_t ke = min(g.K, kb + kChunk);
  if (t < BM) {
    const int64_t m = m0 + t;
    sRowA[t] = m < g.M ? g.baseA + g.rowA[m] : -1;
  } else if (t < BM + BN) {
    const int64_t n = n0 + (t - BM);
    sColB[t - BM] = n < g.N ? g.baseB + g.colB[n] : -1;
  }
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
  const int tx = t & 15, ty = t >> 4;
  for (int64_t k0 = kb; k0 < ke; k0 += BK) {
    __syncthreads();
    if (t < BK) {
      const int64_t k = k0 + t;
      sKA[t] = k < ke ? g.kA[k] : -1;
    } else if (t >= 32 && t < 32 + BK) {
      const int64_t k = k0 + (t - 32);
      sKB[t - 32] = k < ke ? g.kB[k] : -1;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = t + 256 * r;
      int mm, kk;
      if (g.aUnitM) { mm = idx & (BM - 1); kk = idx / BM; }
      else { kk = idx & (BK - 1); mm = idx / BK; }
      const int64_t ro = sRowA[mm], ko = sKA[kk];
      As[kk][mm] = (ro >= 0 && ko >= 0) ? g.A[ro + ko] : 0.0;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = t + 256 * r;
      int nn, kk;
      if (g.bUnitN) { nn = idx & (BN - 1); kk = idx / BN; }
      else { kk = idx & (BK - 1); nn = idx / BK; }
      const int64_t co = sColB[nn], ko = sKB[kk];
      Bs[kk][nn] = (co >= 0 && ko >= 0) ? g.B[co + ko] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int64_t m = m0 + tx + 16 * i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int64_t n = n0 + ty + 16 * j;
      if (n >= g.N) continue;
      if (partial) {
        partial[(int64_t)blockIdx.z * g.M * g.N + m + g.M * n] = acc[i][j];
      } else {
        const int64_t off = g.baseC + g.rowC[m] + g.colC[n];
        double val = g.alpha * acc[i][j];
        if (g.beta != 0.0) val += g.beta * g.C[off];
        g.C[off] = val;
      }
    }
  }
}

__global__ void splitk_reduce_kernel(TableGemm g, int splits, const double *partial) {
  const int64_t MN = g.M * g.N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < MN;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < splits; z++) s += partial[(int64_t)z * MN + e];
    const int64_t m = e % g.M, n = e / g.M;
    const int64_t off = g.baseC + g.rowC[m] + g.colC[n];
    double val = g.alpha * s;
    if (g.beta != 0.0) val += g.beta * g.C[off];
    g.C[off] = val;
  }
}

int choose_splits(const TableGemm &g) {
  const int64_t tiles = ceil_div(g.M, BM) * ceil_div(g.N, BN);
  const int64_t target = 2 * kNumSMs;
  if (tiles >= target || g.K <= 4 * BK) return 1;
  int64_t s = ceil_div(target, tiles);
  s = std::min<int64_t>(s, ceil_div(g.K, 4 * BK));
  // keep the partial buffer below 64 Mi doubles
  while (s > 1 && s * g.M * g.N > (int64_t(64) << 20)) s--;
  return (int)std::max<int64_t>(s, 1);
}

}  // namespace

namespace {
__global__ void dgemv_table_kernel(TableGemm g) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double *__restrict__ B = g.B + g.baseB + g.colB[0];
  for (int64_t m = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < g.M; m += warps) {
    const double *__restrict__ A = g.A + g.baseA + g.rowA[m];
    // four independent partial sums a lane: four loads in flight, fixed order
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int64_t k = lane;
    for (; k + 96 < g.K; k += 128) {
      const int64_t ka0 = g.kA[k], ka1 = g.kA[k + 32], ka2 = g.kA[k + 64], ka3 = g.kA[k + 96];
      const int64_t kb0 = g.kB[k], kb1 = g.kB[k + 32], kb2 = g.kB[k + 64], kb3 = g.kB[k + 96];
      const double a0 = A[ka0], a1 = A[ka1], a2 = A[ka2], a3 = A[ka3];
      const double b0 = B[kb0], b1 = B[kb1], b2 = B[kb2], b3 = B[kb3];
      s0 = fma(a0, b0, s0);
      s1 = fma(a1, b1, s1);
      s2 = fma(a2, b2, s2);
      s3 = fma(a3, b3, s3);
    }
    for (; k < g.K; k += 32) s0 = fma(A[g.kA[k]], B[g.kB[k]], s0);
    double s = (s0 + s1) + (s2 + s3);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) {
      const int64_t off = g.baseC + g.rowC[m] + g.colC[0];
      double val = g.alpha * s;
      if (g.beta != 0.0) val += g.beta * g.C[off];
      g.C[off] = val;
    }
  }
}
}  // namespace

namespace {
// Tables of a skinny contraction seen from its small side (Sm, s indices) and
// its long side (Lg, l indices); C(m, n) at C[cS[m] + cL[n]].
struct SkinnyArgs {
  const double *Sm, *Lg;
  double *C;
  const int64_t *sR, *sK, *lR, *lK, *cS, *cL;
  int s, sp, K;  // sp: s rounded up to 4
  int64_t l;
  float alpha;
  double beta;
};

__device__ __forceinline__ void skinny_out(double *p, float v, double beta) {
  if (beta == 1.0) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"((double)v) : "memory");
  } else if (beta == 0.0) {
    *p = (double)v;
  } else {
    *p = fma(beta, *p, (double)v);
  }
}

// Persistent: each block stages the small operand once (FP32, [k][m]) and its
// warps walk tiles of 32 long indices, one per lane, with the lane's K long
// values in registers; every shared load of four small-side values (a 16-byte
// broadcast) feeds four FMAs.
template <bool STAGE>
__global__ void __launch_bounds__(256) skinny_kernel(SkinnyArgs a) {
  extern __shared__ __align__(16) unsigned char sk_raw[];
  float4 *sS4 = reinterpret_cast<float4 *>(sk_raw);                  // [K][sp / 4]
  int64_t *cSs = reinterpret_cast<int64_t *>(sS4 + a.K * (a.sp / 4));  // [s]
  int64_t *lKs = cSs + a.sp;                                         // [K]
  float *stage = reinterpret_cast<float *>(lKs + kSkinnyMaxK);       // [8][32][33] (STAGE)
  float *sS = reinterpret_cast<float *>(sS4);
  for (int e = threadIdx.x; e < a.K * a.sp; e += blockDim.x) {
    const int m = e % a.sp, k = e / a.sp;
    sS[e] = m < a.s ? (float)a.Sm[a.sR[m] + a.sK[k]] : 0.0f;
  }
  for (int m = threadIdx.x; m < a.s; m += blockDim.x) cSs[m] = a.cS[m];
  for (int k = threadIdx.x; k < a.K; k += blockDim.x) lKs[k] = a.lK[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t tiles = (a.l + 31) / 32;
  for (int64_t t = (int64_t)blockIdx.x * 8 + w; t < tiles; t += (int64_t)gridDim.x * 8) {
    const int64_t n = t * 32 + lane;
    const bool ok = n < a.l;
    const int64_t lr = ok ? a.lR[n] : 0, cl = ok ? a.cL[n] : 0;
    float lv[kSkinnyMaxK];
#pragma unroll
    for (int k = 0; k < kSkinnyMaxK; k++) lv[k] = (ok && k < a.K) ? (float)a.Lg[lr + lKs[k]] : 0.0f;
    if (!STAGE) {
      for (int m4 = 0; m4 < a.sp / 4; m4++) {
        float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
#pragma unroll
        for (int k = 0; k < kSkinnyMaxK; k++) {
          if (k < a.K) {
            const float4 q = sS4[k * (a.sp / 4) + m4];
            c0 = fmaf(q.x, lv[k], c0);
            c1 = fmaf(q.y, lv[k], c1);
            c2 = fmaf(q.z, lv[k], c2);
            c3 = fmaf(q.w, lv[k], c3);
          }
        }
        if (!ok) continue;
        const int m = 4 * m4;
        skinny_out(a.C + cSs[m] + cl, a.alpha * c0, a.beta);
        if (m + 1 < a.s) skinny_out(a.C + cSs[m + 1] + cl, a.alpha * c1, a.beta);
        if (m + 2 < a.s) skinny_out(a.C + cSs[m + 2] + cl, a.alpha * c2, a.beta);
        if (m + 3 < a.s) skinny_out(a.C + cSs[m + 3] + cl, a.alpha * c3, a.beta);
      }
    } else {
      float *st = stage + w * 32 * 33;
      for (int m0 = 0; m0 < a.s; m0 += 32) {
        // this lane's 32 results C(m0 .. m0 + 31, n) into its row of the stage
#pragma unroll
        for (int j4 = 0; j4 < 8; j4++) {
          float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
          const int m4 = m0 / 4 + j4;
          if (4 * m4 < a.sp) {
#pragma unroll
            for (int k = 0; k < kSkinnyMaxK; k++) {
              if (k < a.K) {
                const float4 q = sS4[k * (a.sp / 4) + m4];
                c0 = fmaf(q.x, lv[k], c0);
                c1 = fmaf(q.y, lv[k], c1);
                c2 = fmaf(q.z, lv[k], c2);
                c3 = fmaf(q.w, lv[k], c3);
              }
            }
          }
          st[lane * 33 + 4 * j4] = a.alpha * c0;
          st[lane * 33 + 4 * j4 + 1] = a.alpha * c1;
          st[lane * 33 + 4 * j4 + 2] = a.alpha * c2;
          st[lane * 33 + 4 * j4 + 3] = a.alpha * c3;
        }
        __syncwarp();
        // lanes along the small side: column n' of the tile, rows m0 + lane
        const int m = m0 + lane;
        for (int j = 0; j < 32; j++) {
          const int64_t clj = __shfl_sync(0xffffffffu, cl, j);
          if (t * 32 + j < a.l && m < a.s) skinny_out(a.C + cSs[m] + clj, st[j * 33 + lane], a.beta);
        }
        __syncwarp();
      }
    }
  }
}
}  // namespace

void skinny_table(const TableGemm &g, bool small_is_a, bool stage, cudaStream_t stream) {
  SkinnyArgs a;
  a.Sm = (small_is_a ? g.A + g.baseA : g.B + g.baseB);
  a.Lg = (small_is_a ? g.B + g.baseB : g.A + g.baseA);
  a.C = g.C + g.baseC;
  a.sR = small_is_a ? g.rowA : g.colB;
  a.sK = small_is_a ? g.kA : g.kB;
  a.lR = small_is_a ? g.colB : g.rowA;
  a.lK = small_is_a ? g.kB : g.kA;
  a.cS = small_is_a ? g.rowC : g.colC;
  a.cL = small_is_a ? g.colC : g.rowC;
  const int64_t s = small_is_a ? g.M : g.N, l = small_is_a ? g.N : g.M;
  if (s < 1 || s > kSkinnyMaxS || g.K < 1 || g.K > kSkinnyMaxK || l < 1)
    throw Error(SCESS_ERR_INVALID, "skinny contraction out of range");
  a.s = (int)s;
  a.sp = (int)round_up(s, 4);
  a.K = (int)g.K;
  a.l = l;
  a.alpha = (float)g.alpha;
  a.beta = g.beta;
  const size_t smem = (size_t)a.K * a.sp * sizeof(float) + (size_t)(a.sp + kSkinnyMaxK) * sizeof(int64_t) +
                      (stage ? (size_t)8 * 32 * 33 * sizeof(float) : 0);
  const int64_t tiles = ceil_div(l, 32);
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(tiles, 8), 4 * kNumSMs));
  if (stage) {
    SCESS_CUDA(cudaFuncSetAttribute(skinny_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    skinny_kernel<true><<<blocks, 256, smem, stream>>>(a);
  } else {
    SCESS_CUDA(cudaFuncSetAttribute(skinny_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    skinny_kernel<false><<<blocks, 256, smem, stream>>>(a);
  }
  SCESS_CHECK_LAUNCH();
}

void dgemv_table(const TableGemm &g, cudaStream_t stream) {
  if (g.M <= 0) return;
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(g.M * 32, 256), 16 * kNumSMs);
  dgemv_table_kernel<<<blocks, 256, 0, stream>>>(g);
  SCESS_CHECK_LAUNCH();
}

int64_t dgemm_table_workspace(const TableGemm &g) {
  const int s = choose_splits(g);
  return s > 1 ? s * g.M * g.N : 0;
}

void dgemm_table(const TableGemm &g, double *workspace, cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0) return;
  if (g.K <= 0) {
    // C = beta * C
    TableGemm h = g;
    h.alpha = 0.0;
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>(ceil_div(g.M * g.N, 256), 4096), 256, 0,
                           stream>>>(h, 0, nullptr);
    SCESS_CHECK_LAUNCH();
    return;
  }
  const int splits = choose_splits(g);
  const int64_t kChunk = round_up(ceil_div(g.K, splits), BK);
  const int nz = (int)ceil_div(g.K, kChunk);
  dim3 grid((unsigned)ceil_div(g.M, BM), (unsigned)ceil_div(g.N, BN), (unsigned)nz);
  if (nz > 1) {
    if (!workspace) throw Error(SCESS_ERR_INVALID, "dgemm_table: split-K needs a workspace");
    dgemm_table_kernel<<<grid, 256, 0, stream>>>(g, kChunk, workspace);
    SCESS_CHECK_LAUNCH();
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>(ceil_div(g.M * g.N, 256), 4096), 256, 0,
                           stream>>>(g, nz, workspace);
  } else {
    dgemm_table_kernel<<<grid, 256, 0, stream>>>(g, kChunk, nullptr);
  }
  SCESS_CHECK_LAUNCH();
}

void dgemm_table_bounded(const TableGemm &g, double *workspace, int64_t ws_doubles,
                         cudaStream_t stream) {
  if (g.M <= 0 || g.N <= 0) return;
  const unsigned rblocks = (unsigned)std::min<int64_t>(ceil_div(g.M * g.N, 256), 4096);
  if (g.K <= 0) {
    TableGemm h = g;
    h.alpha = 0.0;
    splitk_reduce_kernel<<<rblocks, 256, 0, stream>>>(h, 0, nullptr);
    SCESS_CHECK_LAUNCH();
    return;
  }
  int splits = choose_splits(g);
  while (splits > 1 && (int64_t)splits * g.M * g.N > ws_doubles) splits--;
  const int64_t kChunk = round_up(ceil_div(g.K, splits), BK);
  const int nz = (int)ceil_div(g.K, kChunk);
  dim3 grid((unsigned)ceil_div(g.M, BM), (unsigned)ceil_div(g.N, BN), (unsigned)nz);
  if (nz > 1) {
    dgemm_table_kernel<<<grid, 256, 0, stream>>>(g, kChunk, workspace);
    SCESS_CHECK_LAUNCH();
    splitk_reduce_kernel<<<rblocks, 256, 0, stream>>>(g, nz, workspace);
  } else {
    dgemm_table_kernel<<<grid, 256, 0, stream>>>(g, kChunk, nullptr);
  }
  SCESS_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------------------------

namespace {

__global__ void permute_add_kernel(PermDesc d, double alpha, const double *__restrict__ X,
                                   double beta, double *__restrict__ Y, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e, xo = 0, yo = 0;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      if (k < d.nd) {
        const int64_t i = r % d.ext[k];
        r /= d.ext[k];
        xo += i * d.xs[k];
        yo += i * d.ys[k];
      }
    }
    double val = alpha * X[xo];
    if (beta != 0.0) val += beta * Y[yo];
    Y[yo] = val;
  }
}

unsigned grid_for(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), 16 * kNumSMs * 8));
}

__global__ void tau_kernel(int64_t o, int64_t v, const double *__restrict__ t1,
                           const double *__restrict__ t2, double s, double *__restrict__ tau) {
  const int64_t n = o * o * v * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % o, j = (e / o) % o, a = (e / (o * o)) % v, b = e / (o * o * v);
    tau[e] = t2[e] + s * t1[i + o * a] * t1[j + o * b];
  }
}

// dtau = tau(t1_0 + dt1, t2_0 + dt2) - tau(t1_0, t2_0)
//      = dt2 + dt1(i,a) t1_1(j,b) + t1_0(i,a) dt1(j,b),  t1_1 = t1_0 + dt1
__global__ void tau_delta_kernel(int64_t o, int64_t v, const double *__restrict__ t1_0,
                                 const double *__restrict__ dt1, const double *__restrict__ dt2,
                                 double *__restrict__ dtau) {
  const int64_t n = o * o * v * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % o, j = (e / o) % o, a = (e / (o * o)) % v, b = e / (o * o * v);
    const int64_t ia = i + o * a, jb = j + o * b;
    dtau[e] = dt2[e] + dt1[ia] * (t1_0[jb] + dt1[jb]) + t1_0[ia] * dt1[jb];
  }
}

// Pairs of the particle ladder's symmetric / antisymmetric form: upper pairs
// p <= q of n labels at u(p, q) = q (q + 1) / 2 + p, strict pairs p < q at
// s(p, q) = q (q - 1) / 2 + p; pu / ps list each pair's (p, q).
__device__ __forceinline__ int64_t upair(int64_t p, int64_t q) { return q * (q + 1) / 2 + p; }
__device__ __forceinline__ int64_t spair(int64_t p, int64_t q) { return q * (q - 1) / 2 + p; }

// Vp(x, k) = V(a,b,c,d) + V(a,b,d,c) (c < d) or V(a,b,c,c) (c = d) for upper
// pairs x = (a,b), k = (c,d); Vm(x, k) = V(a,b,c,d) - V(a,b,d,c) for strict
// pairs.  V(a,b,c,d) = V[a s0 + b s1 + c s2 + d s3].
__global__ void ladder_vpm_kernel(const double *__restrict__ V, int64_t s0, int64_t s1, int64_t s2,
                                  int64_t s3, const int2 *__restrict__ pu, int64_t nu,
                                  const int2 *__restrict__ ps, int64_t ns, double *__restrict__ Vp,
                                  double *__restrict__ Vm) {
  const int64_t total = nu * nu + ns * ns;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < nu * nu) {
      const int2 ab = pu[e % nu], cd = pu[e / nu];
      const int64_t base = ab.x * s0 + ab.y * s1;
      const double v1 = V[base + cd.x * s2 + cd.y * s3];
      Vp[e] = cd.x < cd.y ? v1 + V[base + cd.y * s2 + cd.x * s3] : v1;
    } else {
      const int64_t f = e - nu * nu;
      const int2 ab = ps[f % ns], cd = ps[f / ns];
      const int64_t base = ab.x * s0 + ab.y * s1;
      Vm[f] = V[base + cd.x * s2 + cd.y * s3] - V[base + cd.y * s2 + cd.x * s3];
    }
  }
}

// Tp(y, k) = (tau(i,j,c,d) + tau(i,j,d,c)) / 2 over upper pairs y = (i,j),
// k = (c,d); Tm(y, k) = (tau(i,j,c,d) - tau(i,j,d,c)) / 2 over strict pairs.
__global__ void ladder_tpm_kernel(int64_t o, int64_t v, const double *__restrict__ tau,
                                  const int2 *__restrict__ puo, int64_t nuo,
                                  const int2 *__restrict__ pso, int64_t nso,
                                  const int2 *__restrict__ puv, int64_t nuv,
                                  const int2 *__restrict__ psv, int64_t nsv,
                                  double *__restrict__ Tp, double *__restrict__ Tm) {
  const int64_t total = nuo * nuv + nso * nsv, o2 = o * o, o2v = o2 * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < nuo * nuv) {
      const int2 ij = puo[e % nuo], cd = puv[e / nuo];
      const int64_t b = ij.x + o * ij.y;
      Tp[e] = 0.5 * (tau[b + o2 * cd.x + o2v * cd.y] + tau[b + o2 * cd.y + o2v * cd.x]);
    } else {
      const int64_t f = e - nuo * nuv;
      const int2 ij = pso[f % nso], cd = psv[f / nso];
      const int64_t b = ij.x + o * ij.y;
      Tm[f] = 0.5 * (tau[b + o2 * cd.x + o2v * cd.y] - tau[b + o2 * cd.y + o2v * cd.x]);
    }
  }
}

// R2(i,j,a,b) += Sp(u(i,j), u(a,b)) + sgn Sm(s(i,j), s(a,b)) with the pairs
// sorted and sgn = +1 when (i < j) == (a < b), -1 otherwise (0 when i = j or
// a = b): Sp is symmetric and Sm antisymmetric in each pair.  Sp is
// nuo x nuv, Sm nso x nsv, both column-major.
__global__ void ladder_unpack_kernel(int64_t o, int64_t v, const double *__restrict__ Sp,
                                     const double *__restrict__ Sm, double *__restrict__ R2) {
  const int64_t n = o * o * v * v, nuo = o * (o + 1) / 2, nso = o * (o - 1) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % o, j = (e / o) % o, a = (e / (o * o)) % v, b = e / (o * o * v);
    const int64_t i0 = i < j ? i : j, j0 = i < j ? j : i, a0 = a < b ? a : b, b0 = a < b ? b : a;
    double s = Sp[upair(i0, j0) + nuo * upair(a0, b0)];
    if (i != j && a != b) {
      const double m = Sm[spair(i0, j0) + nso * spair(a0, b0)];
      s += ((i < j) == (a < b)) ? m : -m;
    }
    R2[e] += s;
  }
}

__global__ void denom_kernel(int64_t o, int64_t v, const double *__restrict__ eps,
                             const double *__restrict__ R1, const double *__restrict__ R2,
                             double *__restrict__ t1, double *__restrict__ t2) {
  const int64_t n1 = o * v, n2 = o * o * v * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n1 + n2;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < n1) {
      const int64_t i = e % o, a = e / o;
      t1[e] = R1[e] / (eps[i] - eps[o + a]);
    } else {
      const int64_t x = e - n1;
      const int64_t i = x % o, j = (x / o) % o, a = (x / (o * o)) % v, b = x / (o * o * v);
      // eijab = eia(i,a) + eia(j,b), the reference's association (RCCSD.cpp:331)
      const double d = (eps[i] - eps[o + a]) + (eps[j] - eps[o + b]);
      t2[x] = R2[x] / d;
    }
  }
}

__global__ void plus_transpose_kernel(int64_t o, int64_t v, double alpha,
                                      const double *__restrict__ X, double *__restrict__ out) {
  const int64_t n = o * o * v * v;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % o, j = (e / o) % o, a = (e / (o * o)) % v, b = e / (o * o * v);
    const int64_t et = j + o * i + o * o * b + o * o * v * a;
    out[e] += alpha * (X[e] + X[et]);
  }
}

__global__ void axpby_kernel(int64_t n, double a, const double *__restrict__ x, double b,
                             double *__restrict__ y) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    y[e] = a * x[e] + (b == 0.0 ? 0.0 : b * y[e]);
}

__device__ double block_sum(double v) {
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) r += __shfl_down_sync(0xffffffffu, r, off);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

__global__ void dot_partial_kernel(int64_t n, const double *__restrict__ x,
                                   const double *__restrict__ y, double *__restrict__ partials) {
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    s = fma(x[e], y[e], s);
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void sum_partials_kernel(int np, const double *__restrict__ partials,
                                    double *__restrict__ result) {
  double s = 0.0;
  for (int e = threadIdx.x; e < np; e += blockDim.x) s += partials[e];
  s = block_sum(s);
  if (threadIdx.x == 0) result[0] = s;
}

__global__ void tau_energy_partial_kernel(int64_t o, int64_t v, const double *__restrict__ L,
                                          const double *__restrict__ t1,
                                          const double *__restrict__ t2,
                                          double *__restrict__ partials) {
  const int64_t n = o * o * v * v;
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % o, j = (e / o) % o, a = (e / (o * o)) % v, b = e / (o * o * v);
    const double tau = t2[e] + t1[i + o * a] * t1[j + o * b];
    s = fma(L[e], tau, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// MP2 (RHF.cpp:289-296, 324-340): x = (ia|jb) = g[i si + a sa + j sj + b sb],
// y = (ib|ja) (a and b swapped), eps occupied first.
__global__ void mp2_partial_kernel(int64_t o, int64_t v, const double *__restrict__ g, int64_t si,
                                   int64_t sa, int64_t sj, int64_t sb,
                                   const double *__restrict__ eps, double *__restrict__ partials) {
  const int64_t n = o * v * o * v;
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % o, a = (e / o) % v, j = (e / (o * v)) % o, b = e / (o * v * o);
    const double x = g[i * si + a * sa + j * sj + b * sb];
    const double y = g[i * si + b * sa + j * sj + a * sb];
    s -= x * (2.0 * x - y) / (eps[o + a] + eps[o + b] - eps[i] - eps[j]);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void lincomb_kernel(int64_t n, int nv, const double *const *__restrict__ vecs,
                               const double *__restrict__ coef, double *__restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nv; c++) s += coef[c] * vecs[c][e];
    out[e] = s;
  }
}

__global__ void finite_kernel(int64_t n, const double *__restrict__ x, int *flag) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(x[e])) *flag = 1;
}

}  // namespace

void permute_add(const PermDesc &d, double alpha, const double *X, double beta, double *Y,
                 cudaStream_t stream) {
  int64_t n = 1;
  for (int k = 0; k < d.nd; k++) n *= d.ext[k];
  if (n == 0) return;
  permute_add_kernel<<<grid_for(n), 256, 0, stream>>>(d, alpha, X, beta, Y, n);
  SCESS_CHECK_LAUNCH();
}

void make_tau(int64_t o, int64_t v, const double *t1, const double *t2, double s, double *tau,
              cudaStream_t stream) {
  tau_kernel<<<grid_for(o * o * v * v), 256, 0, stream>>>(o, v, t1, t2, s, tau);
  SCESS_CHECK_LAUNCH();
}

void make_tau_delta(int64_t o, int64_t v, const double *t1_0, const double *dt1,
                    const double *dt2, double *dtau, cudaStream_t stream) {
  tau_delta_kernel<<<grid_for(o * o * v * v), 256, 0, stream>>>(o, v, t1_0, dt1, dt2, dtau);
  SCESS_CHECK_LAUNCH();
}

void ladder_vpm(const double *V, int64_t s0, int64_t s1, int64_t s2, int64_t s3, const int2 *pu,
                int64_t nu, const int2 *ps, int64_t ns, double *Vp, double *Vm,
                cudaStream_t stream) {
  ladder_vpm_kernel<<<grid_for(nu * nu + ns * ns), 256, 0, stream>>>(V, s0, s1, s2, s3, pu, nu, ps,
                                                                    ns, Vp, Vm);
  SCESS_CHECK_LAUNCH();
}

void ladder_tpm(int64_t o, int64_t v, const double *tau, const int2 *puo, int64_t nuo,
                const int2 *pso, int64_t nso, const int2 *puv, int64_t nuv, const int2 *psv,
                int64_t nsv, double *Tp, double *Tm, cudaStream_t stream) {
  ladder_tpm_kernel<<<grid_for(nuo * nuv + nso * nsv), 256, 0, stream>>>(
      o, v, tau, puo, nuo, pso, nso, puv, nuv, psv, nsv, Tp, Tm);
  SCESS_CHECK_LAUNCH();
}

void ladder_unpack(int64_t o, int64_t v, const double *Sp, const double *Sm, double *R2,
                   cudaStream_t stream) {
  ladder_unpack_kernel<<<grid_for(o * o * v * v), 256, 0, stream>>>(o, v, Sp, Sm, R2);
  SCESS_CHECK_LAUNCH();
}

void divide_denominators(int64_t o, int64_t v, const double *eps, const double *R1,
                         const double *R2, double *t1, double *t2, cudaStream_t stream) {
  denom_kernel<<<grid_for(o * v + o * o * v * v), 256, 0, stream>>>(o, v, eps, R1, R2, t1, t2);
  SCESS_CHECK_LAUNCH();
}

void plus_transpose(int64_t o, int64_t v, double alpha, const double *X, double *out,
                    cudaStream_t stream) {
  plus_transpose_kernel<<<grid_for(o * o * v * v), 256, 0, stream>>>(o, v, alpha, X, out);
  SCESS_CHECK_LAUNCH();
}

void axpby(int64_t n, double a, const double *x, double b, double *y, cudaStream_t stream) {
  if (n == 0) return;
  axpby_kernel<<<grid_for(n), 256, 0, stream>>>(n, a, x, b, y);
  SCESS_CHECK_LAUNCH();
}

void dot(int64_t n, const double *x, const double *y, double *partials, double *result,
         cudaStream_t stream) {
  dot_partial_kernel<<<kDotBlocks, 256, 0, stream>>>(n, x, y, partials);
  SCESS_CHECK_LAUNCH();
  sum_partials_kernel<<<1, 1024, 0, stream>>>(kDotBlocks, partials, result);
  SCESS_CHECK_LAUNCH();
}

void linear_combination(int64_t n, int nv, const double *const *vecs, const double *coef,
                        double *out, cudaStream_t stream) {
  lincomb_kernel<<<grid_for(n), 256, 0, stream>>>(n, nv, vecs, coef, out);
  SCESS_CHECK_LAUNCH();
}

void tau_energy(int64_t o, int64_t v, const double *L, const double *t1, const double *t2,
                double *partials, double *result, cudaStream_t stream) {
  tau_energy_partial_kernel<<<kDotBlocks, 256, 0, stream>>>(o, v, L, t1, t2, partials);
  SCESS_CHECK_LAUNCH();
  sum_partials_kernel<<<1, 1024, 0, stream>>>(kDotBlocks, partials, result);
  SCESS_CHECK_LAUNCH();
}

void mp2_energy(int64_t o, int64_t v, const double *g, int64_t si, int64_t sa, int64_t sj,
                int64_t sb, const double *eps, double *partials, double *result,
                cudaStream_t stream) {
  mp2_partial_kernel<<<kDotBlocks, 256, 0, stream>>>(o, v, g, si, sa, sj, sb, eps, partials);
  SCESS_CHECK_LAUNCH();
  sum_partials_kernel<<<1, 1024, 0, stream>>>(kDotBlocks, partials, result);
  SCESS_CHECK_LAUNCH();
}

void check_finite(int64_t n, const double *x, int *flag, cudaStream_t stream) {
  if (n == 0) return;
  finite_kernel<<<grid_for(n), 256, 0, stream>>>(n, x, flag);
  SCESS_CHECK_LAUNCH();
}

}  // namespace scess
