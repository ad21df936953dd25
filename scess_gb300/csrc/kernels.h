// Launch wrappers of the engine's CUDA kernels (all asynchronous on `stream`).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace scess {

// C(m,n) = alpha * sum_k A(m,k) B(k,n) + beta * C(m,n) where every operand
// element is addressed through offset tables: A(m,k) = A[baseA + rowA[m] + kA[k]],
// B(k,n) = B[baseB + colB[n] + kB[k]], C(m,n) = C[baseC + rowC[m] + colC[n]].
// The tables carry any index permutation of the operands, so no transposed
// copy is ever materialised.  Tables are device arrays.
struct TableGemm {
  const double *A = nullptr, *B = nullptr;
  double *C = nullptr;
  const int64_t *rowA = nullptr, *kA = nullptr, *colB = nullptr, *kB = nullptr;
  const int64_t *rowC = nullptr, *colC = nullptr;
  int64_t baseA = 0, baseB = 0, baseC = 0;
  int64_t M = 0, N = 0, K = 0;
  double alpha = 1.0, beta = 0.0;
  int aUnitM = 0;  // A's rows are unit-stride (load mapping hint)
  int bUnitN = 0;  // B's cols are unit-stride
};

// The same contraction over a short K (<= kSkinnyMaxK) with one free side of at
// most kSkinnyMaxS indices (the small side: A's rows when small_is_a, else
// B's columns) and a long other side: HBM-bound, so it runs on the CUDA cores
// in FP32 (operands rounded to FP32, products and the K sum in FP32; the
// result is scaled by alpha in FP32 and added to beta * C in FP64: beta = 1
// by L2 FP64 reductions, beta = 0 by stores, other beta read-modify-write).
// stage: C's unit-stride index is on the small side (stores are then staged
// through shared memory so that lanes run along it).
constexpr int kSkinnyMaxK = 32, kSkinnyMaxS = 256;
void skinny_table(const TableGemm &g, bool small_is_a, bool stage, cudaStream_t stream);

// FP64 matrix-vector form of the same contraction (N == 1), one warp per row,
// deterministic.  Used instead of dgemm_table when N == 1 (or M == 1, swapped).
void dgemv_table(const TableGemm &g, cudaStream_t stream);
// FP64 (DFMA) GEMM. `workspace` (>= ws_doubles) is used for deterministic
// split-K partials; returns the number of doubles it needs when called with
// workspace == nullptr and query == true.
int64_t dgemm_table_workspace(const TableGemm &g);
void dgemm_table(const TableGemm &g, double *workspace, cudaStream_t stream);
// dgemm_table with its split-K partials held to `ws_doubles` doubles of
// `workspace` (fewer splits, down to none, when the usual count does not fit).
void dgemm_table_bounded(const TableGemm &g, double *workspace, int64_t ws_doubles,
                         cudaStream_t stream);

// Y[perm] = alpha * X + beta * Y over an up-to-6-d index space `ext` (column
// major linear order); xs/ys are the element strides of X/Y per index.
struct PermDesc {
  int nd = 0;
  int64_t ext[6] = {1, 1, 1, 1, 1, 1};
  int64_t xs[6] = {0, 0, 0, 0, 0, 0};
  int64_t ys[6] = {0, 0, 0, 0, 0, 0};
};
void permute_add(const PermDesc &d, double alpha, const double *X, double beta, double *Y,
                 cudaStream_t stream);

// tau(i,j,a,b) = t2(i,j,a,b) + s * t1(i,a) t1(j,b)   (column major o,o,v,v)
void make_tau(int64_t o, int64_t v, const double *t1, const double *t2, double s, double *tau,
              cudaStream_t stream);
// dtau = tau(t1_0 + dt1, t2_0 + dt2) - tau(t1_0, t2_0), formed from the changes
// (dt2 + dt1 (x) t1_1 + t1_0 (x) dt1), not as a difference of two taus
void make_tau_delta(int64_t o, int64_t v, const double *t1_0, const double *dt1,
                    const double *dt2, double *dtau, cudaStream_t stream);
// Particle ladder in its symmetric / antisymmetric form (pairs: upper p <= q
// at q(q+1)/2 + p, strict p < q at q(q-1)/2 + p; pu / ps list each pair's
// (p, q)).  ladder_vpm: Vp(x,k) = V(a,b,c,d) + V(a,b,d,c) (c < d) or V(a,b,c,c),
// Vm(x,k) = V(a,b,c,d) - V(a,b,d,c), x = (a,b), k = (c,d), V through strides.
// ladder_tpm: Tp / Tm = (tau(i,j,c,d) +/- tau(i,j,d,c)) / 2 over (i,j), (c,d).
// ladder_unpack: R2(i,j,a,b) += Sp(ij, ab) +/- Sm(ij, ab) (symmetric /
// antisymmetric in each pair), Sp = Tp Vp^T, Sm = Tm Vm^T.
void ladder_vpm(const double *V, int64_t s0, int64_t s1, int64_t s2, int64_t s3, const int2 *pu,
                int64_t nu, const int2 *ps, int64_t ns, double *Vp, double *Vm,
                cudaStream_t stream);
void ladder_tpm(int64_t o, int64_t v, const double *tau, const int2 *puo, int64_t nuo,
                const int2 *pso, int64_t nso, const int2 *puv, int64_t nuv, const int2 *psv,
                int64_t nsv, double *Tp, double *Tm, cudaStream_t stream);
void ladder_unpack(int64_t o, int64_t v, const double *Sp, const double *Sm, double *R2,
                   cudaStream_t stream);
// x[i] = y[i] / d[i] style Jacobi update with on-the-fly denominators:
// t1(i,a) = R1(i,a) / (e_i - e_a); t2(i,j,a,b) = R2 / (e_i + e_j - e_a - e_b).
void divide_denominators(int64_t o, int64_t v, const double *eps, const double *R1,
                         const double *R2, double *t1, double *t2, cudaStream_t stream);
// out(i,j,a,b) = X(i,j,a,b) + X(j,i,b,a) (+= when accumulate)
void plus_transpose(int64_t o, int64_t v, double alpha, const double *X, double *out,
                    cudaStream_t stream);
// y = a * x + b * y (n elements)
void axpby(int64_t n, double a, const double *x, double b, double *y, cudaStream_t stream);
// result[0] = sum_i x[i] * y[i], deterministic (fixed-order two-pass); result is device memory.
void dot(int64_t n, const double *x, const double *y, double *partials, double *result,
         cudaStream_t stream);
constexpr int kDotBlocks = 608;   // 4 x 152 SMs
// out = sum_c coef[c] * vecs[c] for nv vectors of length n (coef on device).
void linear_combination(int64_t n, int nv, const double *const *vecs, const double *coef,
                        double *out, cudaStream_t stream);
// result[0] = sum L(i,j,a,b) * (t2 + t1 t1)(i,j,a,b)  (CorrelationEnergy) deterministic
void tau_energy(int64_t o, int64_t v, const double *L, const double *t1, const double *t2,
                double *partials, double *result, cudaStream_t stream);
// result[0] = E_MP2 = -sum (ia|jb) [2 (ia|jb) - (ib|ja)] / (e_a + e_b - e_i - e_j), with
// (ia|jb) = g[i si + a sa + j sj + b sb] and (ib|ja) the same with a, b swapped;
// deterministic (RHF.cpp:289-296, 324-340)
void mp2_energy(int64_t o, int64_t v, const double *g, int64_t si, int64_t sa, int64_t sj,
                int64_t sb, const double *eps, double *partials, double *result,
                cudaStream_t stream);
// any non-finite value in x -> flag[0] = 1
void check_finite(int64_t n, const double *x, int *flag, cudaStream_t stream);

}  // namespace scess
