// Closed-shell (T) on the GPU (RCCSD_TriplesCorrection, SCESS src/Quantum/CC/RCCSD_T.cpp:17-168).
//
// The virtuals are cut into blocks of nb.  For every block triple A >= B >= C
// the symmetrised connected triples W^{abc}_{ijk} (a in A, b in B, c in C) are
// accumulated in one buffer W[(a,b,c)][i,j,k] by 12 GEMMs: for each of the six
// simultaneous permutations of (ia),(jb),(kc) of Symmetrise (:78-106) the raw
//   w^{xyz}_{i'j'k'} = sum_f P(i',f,x,y) Q(f,j',k',z) - sum_m R(i',j',m,x) t2(m,k',y,z)
// of GetW (:62-68) is one (o nb^2) x (o^2 nb) x v GEMM plus one
// (o^2 nb) x (o nb^2) x o GEMM whose epilogue adds it to W at the permuted
// position, so no Symmetrise scratch copy exists.  An energy kernel then
// evaluates, per unique triple a >= b >= c of the block, V (GetV :70-75),
// Y = W + V, r3(Y), the denominators and the degeneracy (:135-157) and writes
// one partial energy per triple; a fixed-order reduction gives 2 * sum (:167).
//
// FP64 form: DFMA GEMMs straight from the padded FP64 repacks, FP64 W and
// FP64 energy arithmetic.  MIXED form: the same 12 products regroup into three
// sets of four K segments (one grouped tcgen05 launch per block triple) whose
// epilogues add them into one FP32 W with L2 reductions, so that W (nb^3 o^3
// floats, 55 MB at o = 20) stays in L2 between the launch and the energy
// kernel; the operands are packed once per call into FP16 hi/lo rows grouped
// by block.  The energy kernel reads W once, clears it for the next block
// triple and works in FP32 per element with denominators formed from the FP64
// orbital energies in double-float, compensated sums and FP64 per triple.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gemm_tc.h"
#include "triples.h"

namespace scess {

namespace {

__host__ __device__ inline int64_t triple_id(int64_t a, int64_t b, int64_t c) {
  return a * (a + 1) * (a + 2) / 6 + b * (b + 1) / 2 + c;
}

// x / y: fast FP32 division in the mixed form (2 ulp), IEEE division in FP64.
__device__ __forceinline__ double div_fast(double x, double y) { return x / y; }

// One CTA per local triple (a_l, b_l, c_l) of the block triple (A, B, C).
// Shared memory: Y (o^3) then Sbc, Sac, Sab (o^2 each) then t1 columns and the
// occupied orbital energies (o each), all in the arithmetic type CT.
template <typename WT, typename CT>
__global__ void __launch_bounds__(256) triples_energy_kernel(
    const WT *__restrict__ W, int64_t o, int64_t v, int64_t nb, int64_t A, int64_t Bk, int64_t C,
    const double *__restrict__ eps, const double *__restrict__ t1, const double *__restrict__ S,
    double *__restrict__ energies) {
  const int64_t al = blockIdx.x / (nb * nb), bl = (blockIdx.x / nb) % nb, cl = blockIdx.x % nb;
  const int64_t a = A * nb + al, b = Bk * nb + bl, c = C * nb + cl;
  if (a >= v || b >= v || c >= v || b > a || c > b) return;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  __shared__ double red[32];
  const int oo = (int)o, o2 = oo * oo, o3 = o2 * oo;
  // Y(i,j,k) at i + p1 j + p2 k with odd p1, p2: the six permuted reads of r3
  // walk consecutive i with strides 1, p1 or p2, all free of bank conflicts.
  const int p1 = oo | 1, p2 = (p1 * oo) | 1;
  CT *Y = reinterpret_cast<CT *>(sm_raw);
  CT *Sbc = Y + p2 * oo, *Sac = Sbc + o2, *Sab = Sac + o2;
  CT *ta = Sab + o2, *tb = ta + oo, *tc = tb + oo, *eo = tc + oo;
  const WT *Wt = W + ((al * nb + bl) * nb + cl) * (int64_t)o3;
  // S(i,j,a,b) = (ia|jb) at i + o j + o^2 (a + v b)
  for (int e = threadIdx.x; e < o2; e += blockDim.x) {
    Sbc[e] = (CT)S[e + o2 * (b + v * c)];
    Sac[e] = (CT)S[e + o2 * (a + v * c)];
    Sab[e] = (CT)S[e + o2 * (a + v * b)];
  }
  for (int i = threadIdx.x; i < oo; i += blockDim.x) {
    ta[i] = (CT)t1[i + o * a];
    tb[i] = (CT)t1[i + o * b];
    tc[i] = (CT)t1[i + o * c];
    eo[i] = (CT)eps[i];
  }
  __syncthreads();
  // element e = i + o j + o^2 k; thread t visits e = t, t + 256, ... with
  // incrementally maintained (i, j, k)
  const int di = 256 % oo, dj = (256 / oo) % oo, dk = 256 / o2;
  const int i0 = (int)threadIdx.x % oo, j0 = ((int)threadIdx.x / oo) % oo, k0 = (int)threadIdx.x / o2;
  {
    int i = i0, j = j0, k = k0;
    for (int e = threadIdx.x; e < o3; e += 256) {
      // V_ijk = t1_ia (jb|kc) + t1_jb (ia|kc) + t1_kc (ia|jb)   (GetV + Symmetrise)
      Y[i + p1 * j + p2 * k] =
          (CT)Wt[e] + ta[i] * Sbc[j + oo * k] + tb[j] * Sac[i + oo * k] + tc[k] * Sab[i + oo * j];
      i += di;
      int cj = 0;
      if (i >= oo) { i -= oo; cj = 1; }
      j += dj + cj;
      int ck = 0;
      if (j >= oo) { j -= oo; ck = 1; }
      k += dk + ck;
    }
  }
  __syncthreads();
  const CT evirt = (CT)(eps[o + a] + eps[o + b] + eps[o + c]);
  double acc = 0.0;
  CT part = 0;
  int cnt = 0;
  int i = i0, j = j0, k = k0;
  for (int e = threadIdx.x; e < o3; e += 256) {
    // r3(Y) = 4 Y_ijk + Y_kij + Y_jki - 2 Y_kji - 2 Y_ikj - 2 Y_jik               :152-154
    const CT r3 = (CT)4 * Y[i + p1 * j + p2 * k] + Y[k + p1 * i + p2 * j] +
                  Y[j + p1 * k + p2 * i] -
                  (CT)2 * (Y[k + p1 * j + p2 * i] + Y[i + p1 * k + p2 * j] + Y[j + p1 * i + p2 * k]);
    const CT d = ((eo[i] + eo[j]) + eo[k]) - evirt;                              // :155
    part += div_fast((CT)Wt[e] * r3, d);                                           // :156
    if (++cnt == 16) {
      acc += (double)part;
      part = 0;
      cnt = 0;
    }
    i += di;
    int cj = 0;
    if (i >= oo) { i -= oo; cj = 1; }
    j += dj + cj;
    int ck = 0;
    if (j >= oo) { j -= oo; ck = 1; }
    k += dk + ck;
  }
  acc += (double)part;
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += red[q];
    double deg = 1.0;                                                              // :135-139
    if (a == c) deg = 6.0;
    else if (a == b || b == c) deg = 2.0;
    energies[triple_id(a, b, c)] = s / deg;
  }
}

// FP32 copy of S(i, j, a, b) = (ia|jb) for the tensor-core energy kernel.
// out[r ld + c] = (float) x[r cols + c] for c < cols, 0 for cols <= c < ld.
__global__ void to_f32_rows_kernel(const double *__restrict__ x, int64_t rows, int64_t cols,
                                   int64_t ld, float *__restrict__ out) {
  const int64_t n = rows * ld;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ld, c = e - r * ld;
    out[e] = c < cols ? (float)x[r * cols + c] : 0.0f;
  }
}

// Layout of the mixed form's W and of the FP32 copy of S its energy kernel
// reads: rows of o^2 (i, j) pairs are padded to o2p = o^2 rounded up to a
// multiple of 4 floats, so that every k row and every o^3 block starts on a
// 16-byte boundary.  W[((a_l nb + b_l) nb + c_l) o3p + i + o j + o2p k] with
// o3p = o o2p; S as [(a + v b) o2p + i + o j].
__host__ __device__ inline int64_t pad4(int64_t n) { return (n + 3) & ~int64_t(3); }

// FP32 tables of the mixed energy kernel, built once per (T) call: every
// orbital energy as hi + lo (hi = the FP32 rounding of eps, lo = the FP32
// rounding of the remainder) and t1 in FP32.
__global__ void energy_tables_kernel(const double *__restrict__ eps, int64_t n,
                                     const double *__restrict__ t1, int64_t nt1,
                                     float2 *__restrict__ ehl, float *__restrict__ t1f) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n + nt1;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < n) {
      const double x = eps[e];
      const float h = (float)x;
      ehl[e] = make_float2(h, (float)(x - (double)h));
    } else {
      t1f[e - n] = (float)t1[e - n];
    }
  }
}

// Double-float arithmetic in FP32: two_sum gives s + e == a + b exactly
// (Knuth's TwoSum, six FP32 operations, no branch).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Orbits of (i, j, k) under the six orderings, i <= j <= k, for the energy
// kernel: entry = i | j << 8 | k << 16 | m << 24 with m = 0 (three distinct
// indices: the six orderings are six elements), 1 (two equal: each element
// counted twice), 2 (all equal: six times).
std::vector<uint32_t> orbit_table(int64_t o) {
  std::vector<uint32_t> t;
  for (int64_t k = 0; k < o; k++)
    for (int64_t j = 0; j <= k; j++)
      for (int64_t i = 0; i <= j; i++) {
        const uint32_t m = (i == k) ? 2u : ((i == j || j == k) ? 1u : 0u);
        t.push_back((uint32_t)i | (uint32_t)j << 8 | (uint32_t)k << 16 | m << 24);
      }
  return t;
}

// Energy of one block triple in the mixed form.  W^{abc}_{ijk} is the sum of
// the grouped launch's three products: NW = 3 buffers written by the groups
// (W_0[b,c][a], W_1[a,c][b], W_2[a,b][c], as laid out by their tables), or
// NW = 1 buffer the groups reduced into (W[a,b,c]), which this kernel clears
// after reading so that it starts at zero for the next block triple.  Each
// block is o^3 floats in (i, j, k) order, i + o j + o2p k.  One CTA per local
// triple (a_l, b_l, c_l).
//
// Pass 1 (threads own (i, j) pairs and walk k; a pair's loads are all issued
// before any is used): Y = W + V in shared memory, V_ijk = t1_ia (jb|kc) +
// t1_jb (ia|kc) + t1_kc (ia|jb) (GetV, RCCSD_T.cpp:70-75).
// Pass 2 (threads own orbits of (i, j, k)): r3 (:152-154) of an even ordering
// of the orbit is 3 Y + (S_e - 2 S_o), of an odd one 3 Y + (S_o - 2 S_e)
// (S_e, S_o: sums of Y over the even / odd orderings), and the denominator
// (:155) is the same for the whole orbit:
//   sum_orbit W r3(Y) / D = [sum_even W (3 Y + S_e - 2 S_o) + sum_odd W (3 Y + S_o - 2 S_e)] / D,
// one division per orbit instead of six; r3 is formed per ordering before it
// multiplies W (it is a small difference of similar Y values), and W = Y - V
// with V recomputed from the (ia|jb) slices, so that shared memory holds only
// Y and the slices.  D comes from the FP64 orbital energies without FP64
// arithmetic per orbit: every energy is split into FP32 hi + lo, the sum is
// formed in double-float (two_sum) and rounded once.  The orbit sums are
// compensated (Kahan), the sums over the warp double-float, the CTA's FP64.
constexpr int kEnergyMaxO = 32;  // pass 1 keeps a pair's o loads in registers
template <int NW>
__global__ void __launch_bounds__(256) triples_energy_orbit_kernel(
    float *__restrict__ W, int64_t o, int64_t v, int64_t nb, int64_t A, int64_t Bk, int64_t C,
    const float2 *__restrict__ ehl, const float *__restrict__ t1f, const float *__restrict__ S,
    const uint32_t *__restrict__ orbits, int norbits, double *__restrict__ energies) {
  const int al = (int)(blockIdx.x / (nb * nb)), bl = (int)((blockIdx.x / nb) % nb),
            cl = (int)(blockIdx.x % nb);
  const int64_t a = A * nb + al, b = Bk * nb + bl, c = C * nb + cl;
  const int oo = (int)o, o2 = oo * oo;
  const int o2p = (int)pad4(o2), o3p = oo * o2p;
  const int64_t nb3o3 = nb * nb * nb * (int64_t)o3p;
  const float *W0, *W1 = nullptr, *W2 = nullptr;
  if (NW == 3) {
    W0 = W + ((bl * nb + cl) * nb + al) * (int64_t)o3p;
    W1 = W + nb3o3 + ((al * nb + cl) * nb + bl) * (int64_t)o3p;
    W2 = W + 2 * nb3o3 + ((al * nb + bl) * nb + cl) * (int64_t)o3p;
  } else {
    W0 = W + ((al * nb + bl) * nb + cl) * (int64_t)o3p;
  }
  // the next (T) launch may be scheduled once every CTA is here: it does not
  // touch W before this grid is complete
  if (threadIdx.x == 0) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const bool unique = a < v && b < v && c < v && b <= a && c <= b;
  if (!unique) {
    // launched as a programmatic dependent of the grouped GEMM: W is complete
    // and visible only after this wait (no-op for an ordinary launch)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (NW == 1) {  // its block received the launch's sums all the same: clear it
      float4 *w4 = reinterpret_cast<float4 *>(const_cast<float *>(W0));
      for (int e = threadIdx.x; e < o3p / 4; e += blockDim.x) w4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return;
  }
  extern __shared__ __align__(16) unsigned char sm_raw[];
  __shared__ float red_hi[32], red_lo[32];
  __shared__ float s_ev[2];
  // ek[x] = (e_x hi, e_x lo, t1_xc, 0), tab[x] = (t1_xa, t1_xb); Y at
  // i + p1 j + p2 k with odd p1, p2, the (ia|jb) slices at x + p1 y, so that
  // reads along any one index are free of bank conflicts
  const int p1 = oo | 1, p2 = (p1 * oo) | 1;
  float4 *ek = reinterpret_cast<float4 *>(sm_raw);
  float2 *tab = reinterpret_cast<float2 *>(ek + oo);
  float *Y = reinterpret_cast<float *>(tab + oo);
  float *Sbc = Y + p2 * oo, *Sac = Sbc + p1 * oo, *Sab = Sac + p1 * oo;
  const float *S_bc = S + (b + v * c) * o2p, *S_ac = S + (a + v * c) * o2p, *S_ab = S + (a + v * b) * o2p;
  for (int e = threadIdx.x; e < o2; e += blockDim.x) {
    const int x = e % oo, y = e / oo;
    Sbc[x + p1 * y] = S_bc[e];
    Sac[x + p1 * y] = S_ac[e];
    Sab[x + p1 * y] = S_ab[e];
  }
  for (int i = threadIdx.x; i < oo; i += blockDim.x) {
    const float2 e = ehl[i];
    ek[i] = make_float4(e.x, e.y, t1f[i + o * c], 0.f);
    tab[i] = make_float2(t1f[i + o * a], t1f[i + o * b]);
  }
  if (threadIdx.x == 0) {  // e_a + e_b + e_c in double-float
    const float2 ea = ehl[o + a], eb = ehl[o + b], ec = ehl[o + c];
    float s1, e1, s2, e2;
    two_sum(ea.x, eb.x, s1, e1);
    two_sum(s1, ec.x, s2, e2);
    const float lo = (e1 + e2) + ((ea.y + eb.y) + ec.y);
    const float hi = s2 + lo;
    s_ev[0] = hi;
    s_ev[1] = lo - (hi - s2);
  }
  // the tables above come from the call's setup; W from the grouped GEMM just
  // before, complete after this wait
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // pass 1: Y = W + V (loads only; NW = 1 clears W after the barrier below).
  // A pair's o loads are all issued before any is used; the first pair's go
  // out before the barrier that publishes the tables.
  float wr[kEnergyMaxO];
  auto load_pair = [&](int pr) {
#pragma unroll
    for (int k = 0; k < kEnergyMaxO; k++) {
      if (k < oo) {
        const int e = pr + o2p * k;
        wr[k] = W0[e];
        if (NW == 3) wr[k] += W1[e] + W2[e];
      }
    }
  };
  if ((int)threadIdx.x < o2) load_pair(threadIdx.x);
  __syncthreads();
  for (int pr = threadIdx.x; pr < o2; pr += blockDim.x) {
    if (pr != (int)threadIdx.x) load_pair(pr);
    const int i = pr % oo, j = pr / oo;
    const float tai = tab[i].x, tbj = tab[j].y, sab = Sab[i + p1 * j];
    const int yo = i + p1 * j;
#pragma unroll
    for (int k = 0; k < kEnergyMaxO; k++)
      if (k < oo)
        Y[yo + p2 * k] = wr[k] + (tai * Sbc[j + p1 * k] + tbj * Sac[i + p1 * k] + ek[k].z * sab);
  }
  __syncthreads();
  if (NW == 1) {  // the block of W is read: clear it for the next block triple's reductions
    float4 *w4 = reinterpret_cast<float4 *>(const_cast<float *>(W0));
    for (int e = threadIdx.x; e < o3p / 4; e += blockDim.x) w4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // pass 2: orbits
  const float evh = s_ev[0], evl = s_ev[1];
  float sum = 0.0f, comp = 0.0f;
  for (int q = threadIdx.x; q < norbits; q += blockDim.x) {
    const uint32_t code = __ldg(orbits + q);
    const int i = code & 255, j = (code >> 8) & 255, k = (code >> 16) & 255;
    const int m = code >> 24;
    const float2 ti = tab[i], tj = tab[j], tk = tab[k];
    const float4 ei = ek[i], ej = ek[j], ekk = ek[k];
    const int pi = p1 * i, pj = p1 * j, pk = p1 * k, qi = p2 * i, qj = p2 * j, qk = p2 * k;
    // V_xyz = t1_xa Sbc(y,z) + t1_yb Sac(x,z) + t1_zc Sab(x,y) over the orderings
    const float bc_jk = Sbc[j + pk], bc_kj = Sbc[k + pj], bc_ki = Sbc[k + pi],
                bc_ik = Sbc[i + pk], bc_ij = Sbc[i + pj], bc_ji = Sbc[j + pi];
    const float ac_jk = Sac[j + pk], ac_kj = Sac[k + pj], ac_ki = Sac[k + pi],
                ac_ik = Sac[i + pk], ac_ij = Sac[i + pj], ac_ji = Sac[j + pi];
    const float ab_jk = Sab[j + pk], ab_kj = Sab[k + pj], ab_ki = Sab[k + pi],
                ab_ik = Sab[i + pk], ab_ij = Sab[i + pj], ab_ji = Sab[j + pi];
    // even orderings ijk, jki, kij; odd ikj, kji, jik
    const float ye0 = Y[i + pj + qk], ye1 = Y[j + pk + qi], ye2 = Y[k + pi + qj];
    const float yo0 = Y[i + pk + qj], yo1 = Y[k + pj + qi], yo2 = Y[j + pi + qk];
    const float we0 = ye0 - (ti.x * bc_jk + tj.y * ac_ik + ekk.z * ab_ij);
    const float we1 = ye1 - (tj.x * bc_ki + tk.y * ac_ji + ei.z * ab_jk);
    const float we2 = ye2 - (tk.x * bc_ij + ti.y * ac_kj + ej.z * ab_ki);
    const float wo0 = yo0 - (ti.x * bc_kj + tk.y * ac_ij + ej.z * ab_ik);
    const float wo1 = yo1 - (tk.x * bc_ji + tj.y * ac_ki + ei.z * ab_kj);
    const float wo2 = yo2 - (tj.x * bc_ik + ti.y * ac_jk + ekk.z * ab_ji);
    const float Se = (ye0 + ye1) + ye2, So = (yo0 + yo1) + yo2;
    const float ce = Se - 2.0f * So, co = So - 2.0f * Se;                          // :152-154
    float num = we0 * fmaf(3.0f, ye0, ce);
    num = fmaf(we1, fmaf(3.0f, ye1, ce), num);
    num = fmaf(we2, fmaf(3.0f, ye2, ce), num);
    num = fmaf(wo0, fmaf(3.0f, yo0, co), num);
    num = fmaf(wo1, fmaf(3.0f, yo1, co), num);
    num = fmaf(wo2, fmaf(3.0f, yo2, co), num);
    // D = e_i + e_j + e_k - (e_a + e_b + e_c) in double-float, rounded once   :155
    float s1, e1, s2, e2, s3, e3;
    two_sum(ei.x, ej.x, s1, e1);
    two_sum(s1, ekk.x, s2, e2);
    two_sum(s2, -evh, s3, e3);
    const float d = s3 + (((e1 + e2) + e3) + (((ei.y + ej.y) + ekk.y) - evl));
    const float mult = m == 0 ? 1.0f : (m == 1 ? 0.5f : (1.0f / 6.0f));
    const float term = __fdividef(num * mult, d) - comp;                           // :156
    const float t = sum + term;
    comp = (t - sum) - term;
    sum = t;
  }
  // warp sums in double-float, the CTA's in FP64
  float acc_hi = sum, acc_lo = -comp;
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, acc_hi, off);
    const float ol = __shfl_down_sync(0xffffffffu, acc_lo, off);
    float h, e;
    two_sum(acc_hi, oh, h, e);
    acc_hi = h;
    acc_lo += e + ol;
  }
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  if (lane == 0) {
    red_hi[wi] = acc_hi;
    red_lo[wi] = acc_lo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double total = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) total += (double)red_hi[q] + (double)red_lo[q];
    double deg = 1.0;                                                               // :135-139
    if (a == c) deg = 6.0;
    else if (a == b || b == c) deg = 2.0;
    energies[triple_id(a, b, c)] = total / deg;
  }
}

__global__ void sum_energies_kernel(int64_t n, const double *__restrict__ e, double *out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += e[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
    out[0] = 2.0 * t;                                                              // :167
  }
}

// Offset table over a list of (extent, stride) dims, first fastest:
// entry e = sum_d i_d stride_d for e = i_0 + ext_0 (i_1 + ext_1 (...)).  Kept
// as a spec and filled on the device (DevTables::build).
struct TableSpec {
  int nd = 0;
  int64_t ext[6] = {1, 1, 1, 1, 1, 1}, str[6] = {0, 0, 0, 0, 0, 0};
  int64_t size() const {
    int64_t n = 1;
    for (int d = 0; d < nd; d++) n *= ext[d];
    return n;
  }
};

TableSpec table(std::initializer_list<std::pair<int64_t, int64_t>> dims) {
  TableSpec t;
  if (dims.size() > 6) throw Error(SCESS_ERR_INVALID, "offset table: too many dims");
  for (auto &d : dims) {
    t.ext[t.nd] = d.first;
    t.str[t.nd] = d.second;
    t.nd++;
  }
  return t;
}

constexpr int kMaxTables = 24;
struct TableBatch {
  int nt = 0;
  int64_t start[kMaxTables + 1] = {};
  TableSpec spec[kMaxTables];
  int64_t *out = nullptr;
};

__global__ void fill_tables_kernel(const __grid_constant__ TableBatch b) {
  const int64_t total = b.start[b.nt];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int t = 0;
    while (e >= b.start[t + 1]) t++;
    const TableSpec &sp = b.spec[t];
    int64_t r = e - b.start[t], off = 0;
    for (int d = 0; d < sp.nd; d++) {
      const int64_t q = r / sp.ext[d];
      off += (r - q * sp.ext[d]) * sp.str[d];
      r = q;
    }
    b.out[e] = off;
  }
}

struct DevTables {
  DevMem mem;
  std::vector<const int64_t *> ptr;
  // One allocation, filled by one kernel per kMaxTables tables on ctx's stream.
  void build(Ctx &ctx, const std::vector<TableSpec> &ts) {
    size_t tot = 0;
    for (auto &t : ts) tot += (size_t)t.size();
    mem.alloc(std::max<size_t>(tot, 1) * sizeof(int64_t));
    ptr.clear();
    size_t off = 0;
    for (size_t i0 = 0; i0 < ts.size(); i0 += kMaxTables) {
      TableBatch b;
      b.out = mem.as<int64_t>() + off;
      b.nt = (int)std::min<size_t>(kMaxTables, ts.size() - i0);
      int64_t n = 0;
      for (int t = 0; t < b.nt; t++) {
        b.spec[t] = ts[i0 + t];
        b.start[t] = n;
        ptr.push_back(mem.as<int64_t>() + off + n);
        n += ts[i0 + t].size();
      }
      b.start[b.nt] = n;
      if (n > 0) {
        fill_tables_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), 8 * kNumSMs), 256, 0,
                             ctx.stream>>>(b);
        SCESS_CHECK_LAUNCH();
      }
      off += (size_t)n;
    }
  }
};

// The six simultaneous permutations of Symmetrise, as position maps: the raw
// term w^{u[p0] u[p1] u[p2]}_{w[p0] w[p1] w[p2]} feeds W^{abc}_{ijk}.
const int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

int choose_nb(int64_t o, int64_t v, size_t welem_bytes, size_t budget) {
  const int64_t forced = tune_value("t_nb", 0);  // block size override (tests, tuning)
  if (forced >= 1) return (int)std::min<int64_t>(forced, v);
  const double o3 = (double)o * o * o;
  int nb = (int)std::floor(std::cbrt((double)budget / (welem_bytes * o3)));
  nb = std::max(1, std::min<int>(nb, (int)v));
  // balance the blocks over v
  const int64_t nblk = ceil_div(v, nb);
  nb = (int)ceil_div(v, nblk);
  return nb;
}

// W tables: W's unit-stride index i is kept first on the lane side (GEMM rows)
// or on the per-thread side (GEMM columns) of every epilogue: when i is the k'
// of a permutation the Q operand is taken in (k', j', z) column order, when it
// is the j' of an R product the R operand is taken in (j', i', x) row order.
bool q_swapped(const int *pi) { return pi[2] == 0; }
bool r_swapped(const int *pi) { return pi[1] == 0; }

// FP64 repacks of RCCSD_T.cpp:30-56 (virtuals padded to vp) and the offset
// tables of the block-triple GEMMs: per permutation p the W rows / columns of
// its P.Q and R.t2 products (dt.ptr[4p .. 4p+3]), then the operand tables
// (dt.ptr[kOperand + 0 .. 9]).
struct TriplesSetup {
  int64_t o = 0, v = 0, N = 0, nb = 0, NB = 0, vp = 0;
  DTensor P, Qt, Rt, T2p;
  DTensor S;  // S(i,j,a,b) = (ia|jb), o x o x v x v
  DevTables dt;
  size_t kOperand = 0;
  // integrals from the eri (views) or, when d_B is given, from the DF factors
  // B (naux x N x N): P, R, S are single B.B contractions (be: FP64 or tensor
  // cores), so the N^4 eri is never formed
  void build(Ctx &ctx, const double *d_eri, const double *d_t2, const double *d_B = nullptr,
             int64_t naux = 0, Backend be = Backend::FP64);
  int64_t Mpq() const { return o * nb * nb; }
  int64_t Npq() const { return o * o * nb; }
  int64_t Mr() const { return o * o * nb; }
  int64_t Nr() const { return o * nb * nb; }
};

void TriplesSetup::build(Ctx &ctx, const double *d_eri, const double *d_t2, const double *d_B,
                         int64_t naux, Backend be) {
  cudaStream_t s = ctx.stream;
  const int64_t o2 = o * o, o3 = o2 * o, N2 = N * N, N3 = N2 * N;
  S = DTensor({o, o, v, v});
  // Zero-padded FP64 repacks (RCCSD_T.cpp:30-56), virtual indices padded to vp.
  P = DTensor({o, v, vp, vp});   // P(i,f,a,b) = (ia|bf) = eri(i, o+b, o+a, o+f)
  Qt = DTensor({v, o, o, vp});   // Q(f,j,k,c) = t2(k,j,c,f)
  Rt = DTensor({o, o, o, vp});   // R(i,j,m,a) = (ia|mj) = eri(i, m, o+a, j)
  T2p = DTensor({o, o, vp, vp}); // t2(m,k,b,c)
  SCESS_CUDA(cudaMemsetAsync(P.p(), 0, P.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(Qt.p(), 0, Qt.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(Rt.p(), 0, Rt.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(T2p.p(), 0, T2p.size() * sizeof(double), s));
  {
    TV Pv = P.v;
    Pv.ext[2] = v;
    Pv.ext[3] = v;
    TV Rv = Rt.v;
    Rv.ext[3] = v;
    if (d_B) {
      // (pq|rs) = sum_Q B(Q,p,q) B(Q,r,s): P(i,f,a,b) = (ia|bf), R(i,j,m,a) = (ia|mj),
      // S(i,j,a,b) = (ia|jb)
      auto bview = [&](int64_t p0, int64_t q0, int64_t np, int64_t nq) {
        TV b;
        b.p = const_cast<double *>(d_B) + naux * p0 + naux * N * q0;
        b.nd = 3;
        const int64_t be3[3] = {naux, np, nq}, bs3[3] = {1, naux, naux * N};
        std::memcpy(b.ext, be3, sizeof(be3));
        std::memcpy(b.str, bs3, sizeof(bs3));
        return b;
      };
      const TV Bov = bview(0, o, o, v), Bvv = bview(o, o, v, v), Boo = bview(0, 0, o, o);
      einsum(ctx, "Qia,Qbf->ifab", 1.0, Bov, Bvv, 0.0, Pv, be);
      einsum(ctx, "Qia,Qmj->ijma", 1.0, Bov, Boo, 0.0, Rv, be);
      einsum(ctx, "Qia,Qjb->ijab", 1.0, Bov, Bov, 0.0, S.v, be);
    } else {
      TV e;  // (i, b, a, f) -> eri(i, o+b, o+a, o+f)
      e.p = const_cast<double *>(d_eri) + o * N + o * N2 + o * N3;
      e.nd = 4;
      int64_t ee[4] = {o, v, v, v}, es[4] = {1, N, N2, N3};
      std::memcpy(e.ext, ee, sizeof(ee));
      std::memcpy(e.str, es, sizeof(es));
      permute(ctx, "ibaf->ifab", 1.0, e, 0.0, Pv);
      TV r;  // (i, m, a, j) -> eri(i, m, o+a, j)
      r.p = const_cast<double *>(d_eri) + o * N2;
      r.nd = 4;
      int64_t re[4] = {o, o, v, o}, rs[4] = {1, N, N2, N3};
      std::memcpy(r.ext, re, sizeof(re));
      std::memcpy(r.str, rs, sizeof(rs));
      permute(ctx, "imaj->ijma", 1.0, r, 0.0, Rv);
      TV sv = r;  // (i, j, a, b) -> eri(i, j, o+a, o+b)
      sv.p = const_cast<double *>(d_eri) + o * N2 + o * N3;
      sv.ext[2] = v;
      sv.ext[3] = v;
      permute(ctx, "ijab->ijab", 1.0, sv, 0.0, S.v);
    }
    const TV t2 = cm(const_cast<double *>(d_t2), {o, o, v, v});
    TV Qv = Qt.v;
    Qv.ext[3] = v;
    permute(ctx, "kjcf->fjkc", 1.0, t2, 0.0, Qv);
    TV Tv = T2p.v;
    Tv.ext[2] = v;
    Tv.ext[3] = v;
    permute(ctx, "mkbc->mkbc", 1.0, t2, 0.0, Tv);
  }

  // Output positions in W[(a_l,b_l,c_l)][i,j,k]: strides of (a_l,b_l,c_l) and (i,j,k).
  const int64_t su[3] = {o3 * nb * nb, o3 * nb, o3};
  const int64_t sw[3] = {1, o, o2};
  // Tables per permutation: PQ rows/cols and R rows/cols in W.  W's unit-stride
  // index i is kept first on the lane side (GEMM rows) or on the per-thread side
  // (GEMM columns) of every epilogue: when i is the k' of a permutation the Q
  // operand is taken in (k', j', z) column order, when it is the j' of an R
  // product the R operand is taken in (j', i', x) row order.
  std::vector<TableSpec> ts;
  for (int p = 0; p < 6; p++) {
    const int *pi = kPerm[p];
    ts.push_back(table({{o, sw[pi[0]]}, {nb, su[pi[0]]}, {nb, su[pi[1]]}}));      // PQ rows (i',x,y)
    if (q_swapped(pi))
      ts.push_back(table({{o, sw[pi[2]]}, {o, sw[pi[1]]}, {nb, su[pi[2]]}}));     // PQ cols (k',j',z)
    else
      ts.push_back(table({{o, sw[pi[1]]}, {o, sw[pi[2]]}, {nb, su[pi[2]]}}));     // PQ cols (j',k',z)
    if (r_swapped(pi))
      ts.push_back(table({{o, sw[pi[1]]}, {o, sw[pi[0]]}, {nb, su[pi[0]]}}));     // R rows (j',i',x)
    else
      ts.push_back(table({{o, sw[pi[0]]}, {o, sw[pi[1]]}, {nb, su[pi[0]]}}));     // R rows (i',j',x)
    ts.push_back(table({{o, sw[pi[2]]}, {nb, su[pi[1]]}, {nb, su[pi[2]]}}));      // R cols (k',y,z)
  }
  kOperand = ts.size();
  // operand tables (FP64 path): P rows (i',x,y), f; Q cols (j',k',z), f; R rows, m; t2 cols, m
  ts.push_back(table({{o, 1}, {nb, o * v}, {nb, o * v * vp}}));                  // +0: P rows
  ts.push_back(table({{v, o}}));                                                 // +1: P k (f)
  ts.push_back(table({{o, v}, {o, v * o}, {nb, v * o2}}));                       // +2: Q cols (j,k,z)
  ts.push_back(table({{v, 1}}));                                                 // +3: Q k (f)
  ts.push_back(table({{o, 1}, {o, o}, {nb, o3}}));                               // +4: R rows (i,j,x)
  ts.push_back(table({{o, o2}}));                                                // +5: R k (m)
  ts.push_back(table({{o, o}, {nb, o2}, {nb, o2 * vp}}));                        // +6: t2 cols
  ts.push_back(table({{o, 1}}));                                                 // +7: t2 k (m)
  ts.push_back(table({{o, v * o}, {o, v}, {nb, v * o2}}));                       // +8: Q cols (k,j,z)
  ts.push_back(table({{o, o}, {o, 1}, {nb, o3}}));                               // +9: R rows (j,i,x)
  dt.build(ctx, ts);
}

// The 12 FP64 GEMMs of block triple U = (A, B, C): W[(a_l,b_l,c_l)][i,j,k] =
// sum over the six permutations of the raw P.Q - R.t2 product (GetW,
// RCCSD_T.cpp:62-68), each added at its permuted position (Symmetrise :78-106).
// tc: the same GEMMs on the tensor cores (TcEngine::table_gemm).
void w_block_fp64(Ctx &ctx, const TriplesSetup &T, const int64_t U[3], double *W, double *ws,
                  bool tc = false) {
  cudaStream_t s = ctx.stream;
  const int64_t o = T.o, v = T.v, nb = T.nb, vp = T.vp, o2 = o * o, o3 = o2 * o;
  for (int p = 0; p < 6; p++) {
    const int *pi = kPerm[p];
    const int64_t X = U[pi[0]], Yb = U[pi[1]], Z = U[pi[2]];
    const int64_t *rowPQ = T.dt.ptr[4 * p + 0], *colPQ = T.dt.ptr[4 * p + 1];
    const int64_t *rowR = T.dt.ptr[4 * p + 2], *colR = T.dt.ptr[4 * p + 3];
    TableGemm g;
    g.A = T.P.p();
    g.B = T.Qt.p();
    g.C = W;
    g.rowA = T.dt.ptr[T.kOperand + 0];
    g.kA = T.dt.ptr[T.kOperand + 1];
    g.colB = T.dt.ptr[T.kOperand + (q_swapped(pi) ? 8 : 2)];
    g.kB = T.dt.ptr[T.kOperand + 3];
    g.rowC = rowPQ;
    g.colC = colPQ;
    g.baseA = o * v * (X * nb) + o * v * vp * (Yb * nb);
    g.baseB = v * o2 * (Z * nb);
    g.M = T.Mpq();
    g.N = T.Npq();
    g.K = v;
    g.alpha = 1.0;
    g.beta = p == 0 ? 0.0 : 1.0;
    g.aUnitM = 1;
    g.bUnitN = 0;
    if (tc) {
      ctx.tensor_cores().table_gemm(g, "triples_w");
    } else {
      TimedScope ts(ctx.timer, "dgemm_table", 2.0 * g.M * g.N * g.K, 0.0, s);
      dgemm_table(g, ws, s);
    }
    TableGemm h;
    h.A = T.Rt.p();
    h.B = T.T2p.p();
    h.C = W;
    h.rowA = T.dt.ptr[T.kOperand + (r_swapped(pi) ? 9 : 4)];
    h.kA = T.dt.ptr[T.kOperand + 5];
    h.colB = T.dt.ptr[T.kOperand + 6];
    h.kB = T.dt.ptr[T.kOperand + 7];
    h.rowC = rowR;
    h.colC = colR;
    h.baseA = o3 * (X * nb);
    h.baseB = o2 * (Yb * nb) + o2 * vp * (Z * nb);
    h.M = T.Mr();
    h.N = T.Nr();
    h.K = o;
    h.alpha = -1.0;
    h.beta = 1.0;
    h.aUnitM = r_swapped(pi) ? 0 : 1;
    h.bUnitN = 0;
    if (tc) {
      ctx.tensor_cores().table_gemm(h, "triples_w");
    } else {
      TimedScope ts(ctx.timer, "dgemm_table", 2.0 * h.M * h.N * h.K, 0.0, s);
      dgemm_table(h, ws, s);
    }
  }
}

// Gradient of the block triple's energy with respect to its W and V (FP64).
// With L = r3 (a symmetric linear map over the six orderings of (i,j,k): the
// two cyclic shifts are each other's transposes, the three swaps are their own)
// and the triple's term E_abc = (2/deg) sum W L(W + V) / D:
//   dE/dW = (2/deg) [L(Y)/D + L(W/D)],   dE/dV = (2/deg) L(W/D),   Y = W + V.
// G (W's layout) receives gE dE/dW, zero for triples outside a >= b >= c; dE/dV
// flows into t1 and the (ia|jb) slices S (o x o x v x v) through
// V_ijk = t1_ia S(j,k,b,c) + t1_jb S(i,k,a,c) + t1_kc S(i,j,a,b) (:70-75, :132)
// with global FP64 atomics.  Also writes the triple's energy like the energy
// kernel.  One CTA per (a_l, b_l, c_l); threads own (i, j) pairs and walk k.
__global__ void __launch_bounds__(256) triples_grad_kernel(
    const double *__restrict__ W, double *__restrict__ G, int64_t o, int64_t v, int64_t nb,
    int64_t A, int64_t Bk, int64_t C, const double *__restrict__ eps,
    const double *__restrict__ t1, const double *__restrict__ Sg, double gE,
    double *__restrict__ energies, double *__restrict__ g_t1, double *__restrict__ g_S) {
  const int64_t al = blockIdx.x / (nb * nb), bl = (blockIdx.x / nb) % nb, cl = blockIdx.x % nb;
  const int64_t a = A * nb + al, b = Bk * nb + bl, c = C * nb + cl;
  const int oo = (int)o, o2 = oo * oo, o3 = o2 * oo;
  const double *Wt = W + ((al * nb + bl) * nb + cl) * (int64_t)o3;
  double *Gt = G + ((al * nb + bl) * nb + cl) * (int64_t)o3;
  if (a >= v || b >= v || c >= v || b > a || c > b) {
    for (int e = threadIdx.x; e < o3; e += blockDim.x) Gt[e] = 0.0;
    return;
  }
  extern __shared__ __align__(16) unsigned char sm_raw[];
  __shared__ double red[32];
  const int p1 = oo | 1, p2 = (p1 * oo) | 1;
  double *Y = reinterpret_cast<double *>(sm_raw);
  double *Sbc = Y + p2 * oo, *Sac = Sbc + o2, *Sab = Sac + o2;
  double *gSbc = Sab + o2, *gSac = gSbc + o2;
  double *ta = gSac + o2, *tb = ta + oo, *tc = tb + oo, *eo = tc + oo;
  double *gta = eo + oo, *gtb = gta + oo, *gtc = gtb + oo;
  for (int e = threadIdx.x; e < o2; e += blockDim.x) {
    Sbc[e] = Sg[e + o2 * (b + v * c)];
    Sac[e] = Sg[e + o2 * (a + v * c)];
    Sab[e] = Sg[e + o2 * (a + v * b)];
    gSbc[e] = 0.0;
    gSac[e] = 0.0;
  }
  for (int i = threadIdx.x; i < oo; i += blockDim.x) {
    ta[i] = t1[i + o * a];
    tb[i] = t1[i + o * b];
    tc[i] = t1[i + o * c];
    eo[i] = eps[i];
    gta[i] = gtb[i] = gtc[i] = 0.0;
  }
  __syncthreads();
  const double evirt = eps[o + a] + eps[o + b] + eps[o + c];
  double deg = 1.0;                                                                 // :135-139
  if (a == c) deg = 6.0;
  else if (a == b || b == c) deg = 2.0;
  const double fac = gE * 2.0 / deg;
  auto L = [&](int i, int j, int k) {  // r3 at (i,j,k) of the array in Y   :152-154
    return 4.0 * Y[i + p1 * j + p2 * k] + Y[k + p1 * i + p2 * j] + Y[j + p1 * k + p2 * i] -
           2.0 * (Y[k + p1 * j + p2 * i] + Y[i + p1 * k + p2 * j] + Y[j + p1 * i + p2 * k]);
  };
  // Y = W + V
  for (int pr = threadIdx.x; pr < o2; pr += blockDim.x) {
    const int i = pr % oo, j = pr / oo;
    for (int k = 0; k < oo; k++)
      Y[i + p1 * j + p2 * k] = Wt[pr + o2 * k] + ta[i] * Sbc[j + oo * k] + tb[j] * Sac[i + oo * k] +
                               tc[k] * Sab[pr];
  }
  __syncthreads();
  // G = fac L(Y)/D; energy term W L(Y)/D
  double acc = 0.0;
  for (int pr = threadIdx.x; pr < o2; pr += blockDim.x) {
    const int i = pr % oo, j = pr / oo;
    for (int k = 0; k < oo; k++) {
      const double d = ((eo[i] + eo[j]) + eo[k]) - evirt;                           // :155
      const double ly = L(i, j, k) / d;
      Gt[pr + o2 * k] = fac * ly;
      acc += Wt[pr + o2 * k] * ly;                                                  // :156
    }
  }
  __syncthreads();
  // Y = W/D
  for (int pr = threadIdx.x; pr < o2; pr += blockDim.x) {
    const int i = pr % oo, j = pr / oo;
    for (int k = 0; k < oo; k++)
      Y[i + p1 * j + p2 * k] = Wt[pr + o2 * k] / (((eo[i] + eo[j]) + eo[k]) - evirt);
  }
  __syncthreads();
  // G += fac L(W/D); dE/dV = fac L(W/D) into t1 and S
  for (int pr = threadIdx.x; pr < o2; pr += blockDim.x) {
    const int i = pr % oo, j = pr / oo;
    double sa = 0.0, sb = 0.0, sab = 0.0;
    for (int k = 0; k < oo; k++) {
      const double gv = fac * L(i, j, k);
      Gt[pr + o2 * k] += gv;
      sa += gv * Sbc[j + oo * k];      // t1_ia (jb|kc)
      sb += gv * Sac[i + oo * k];      // t1_jb (ia|kc)
      sab += gv * tc[k];               // (ia|jb) t1_kc
      atomicAdd(&gtc[k], gv * Sab[pr]);
      atomicAdd(&gSbc[j + oo * k], gv * ta[i]);
      atomicAdd(&gSac[i + oo * k], gv * tb[j]);
    }
    atomicAdd(&gta[i], sa);
    atomicAdd(&gtb[j], sb);
    atomicAdd(&g_S[pr + o2 * (a + v * b)], sab);  // (i,j) owned by this thread
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  if (lane == 0) red[wi] = acc;
  __syncthreads();
  for (int e = threadIdx.x; e < o2; e += blockDim.x) {
    atomicAdd(&g_S[e + o2 * (b + v * c)], gSbc[e]);
    atomicAdd(&g_S[e + o2 * (a + v * c)], gSac[e]);
  }
  for (int i = threadIdx.x; i < oo; i += blockDim.x) {
    atomicAdd(&g_t1[i + o * a], gta[i]);
    atomicAdd(&g_t1[i + o * b], gtb[i]);
    atomicAdd(&g_t1[i + o * c], gtc[i]);
  }
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) sum += red[q];
    energies[triple_id(a, b, c)] = sum / deg;
  }
}

// Transposed GEMMs of w_block_fp64 for block triple U: with G = dE/dW,
//   gP  += G Q,   gQ  += G^T P,   gR -= G' t2,   gt2 -= G'^T R
// per permutation, G read through that permutation's W tables.
// tc: the same GEMMs on the tensor cores (TcEngine::table_gemm).
void g_block_fp64(Ctx &ctx, const TriplesSetup &T, const int64_t U[3], const double *G, double *gP,
                  double *gQt, double *gRt, double *gT2p, bool integrals, double *ws,
                  bool tc = false) {
  cudaStream_t s = ctx.stream;
  const int64_t o = T.o, v = T.v, nb = T.nb, vp = T.vp, o2 = o * o, o3 = o2 * o;
  const size_t K0 = T.kOperand;
  auto run = [&](TableGemm &g) {
    if (tc) {
      ctx.tensor_cores().table_gemm(g, "triples_vjp");
      return;
    }
    TimedScope ts(ctx.timer, "dgemm_table", 2.0 * g.M * g.N * g.K, 0.0, s);
    dgemm_table(g, ws, s);
  };
  for (int p = 0; p < 6; p++) {
    const int *pi = kPerm[p];
    const int64_t X = U[pi[0]], Yb = U[pi[1]], Z = U[pi[2]];
    const int64_t *rowPQ = T.dt.ptr[4 * p + 0], *colPQ = T.dt.ptr[4 * p + 1];
    const int64_t *rowR = T.dt.ptr[4 * p + 2], *colR = T.dt.ptr[4 * p + 3];
    const int64_t *qcols = T.dt.ptr[K0 + (q_swapped(pi) ? 8 : 2)];
    const int64_t *rrows = T.dt.ptr[K0 + (r_swapped(pi) ? 9 : 4)];
    const int64_t baseP = o * v * (X * nb) + o * v * vp * (Yb * nb), baseQ = v * o2 * (Z * nb);
    const int64_t baseR = o3 * (X * nb), baseT = o2 * (Yb * nb) + o2 * vp * (Z * nb);
    if (integrals) {  // gP(m, f) += sum_n G(m, n) Q(n, f)
      TableGemm g;
      g.A = G; g.rowA = rowPQ; g.kA = colPQ;
      g.B = T.Qt.p(); g.colB = T.dt.ptr[K0 + 3]; g.kB = qcols; g.baseB = baseQ;
      g.C = gP; g.rowC = T.dt.ptr[K0 + 0]; g.colC = T.dt.ptr[K0 + 1]; g.baseC = baseP;
      g.M = T.Mpq(); g.N = v; g.K = T.Npq(); g.alpha = 1.0; g.beta = 1.0;
      run(g);
    }
    {  // gQ(n, f) += sum_m G(m, n) P(m, f)
      TableGemm g;
      g.A = G; g.rowA = colPQ; g.kA = rowPQ;
      g.B = T.P.p(); g.colB = T.dt.ptr[K0 + 1]; g.kB = T.dt.ptr[K0 + 0]; g.baseB = baseP;
      g.C = gQt; g.rowC = qcols; g.colC = T.dt.ptr[K0 + 3]; g.baseC = baseQ;
      g.M = T.Npq(); g.N = v; g.K = T.Mpq(); g.alpha = 1.0; g.beta = 1.0;
      run(g);
    }
    if (integrals) {  // gR(r, m) -= sum_n G(r, n) t2(n, m)
      TableGemm g;
      g.A = G; g.rowA = rowR; g.kA = colR;
      g.B = T.T2p.p(); g.colB = T.dt.ptr[K0 + 7]; g.kB = T.dt.ptr[K0 + 6]; g.baseB = baseT;
      g.C = gRt; g.rowC = rrows; g.colC = T.dt.ptr[K0 + 5]; g.baseC = baseR;
      g.M = T.Mr(); g.N = o; g.K = T.Nr(); g.alpha = -1.0; g.beta = 1.0;
      run(g);
    }
    {  // gt2(n, m) -= sum_r G(r, n) R(r, m)
      TableGemm g;
      g.A = G; g.rowA = colR; g.kA = rowR;
      g.B = T.Rt.p(); g.colB = T.dt.ptr[K0 + 5]; g.kB = rrows; g.baseB = baseR;
      g.C = gT2p; g.rowC = T.dt.ptr[K0 + 6]; g.colC = T.dt.ptr[K0 + 7]; g.baseC = baseT;
      g.M = T.Nr(); g.N = o; g.K = T.Mr(); g.alpha = -1.0; g.beta = 1.0;
      run(g);
    }
  }
}

// Block size of the grouped tensor-core form: GEMM rows (u, x_l) = o nb fill
// the 128-row tiles well, the padded virtual range vp = NB nb stays close to v,
// and W (nb^3 o^3 floats per buffer) stays within 64 MiB a buffer; ties go to
// the larger block (fewer, larger launches).  The tuning key t_nb overrides it.
int choose_nb_grouped(int64_t o, int64_t v) {
  const int64_t forced = tune_value("t_nb", 0);
  if (forced >= 1) return (int)std::min<int64_t>(forced, v);
  int best = 1;
  double best_score = -1.0;
  const double o3 = (double)o * o * o;
  for (int nb = 1; nb <= std::min<int64_t>(v, 64); nb++) {
    if (nb > 1 && (double)nb * nb * nb * o3 * 4.0 > double(64 << 20)) break;
    const double rows = (double)o * nb;
    const double effM = rows / (128.0 * std::ceil(rows / 128.0));
    const double vp = (double)ceil_div(v, nb) * nb;
    const double effV = std::pow((double)v / vp, 3.0);
    const double score = effM * effV;
    if (score >= best_score * (1.0 - 1e-9)) {
      best = nb;
      best_score = std::max(score, best_score);
    }
  }
  return best;
}

}  // namespace

double rccsd_triples(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t o, const double *d_eps,
                     const double *d_t1, const double *d_t2, bool mixed, const Control &ctl,
                     TriplesStats *stats, const double *d_B, int64_t naux) {
  const int64_t v = nmo - o, N = nmo;
  cudaStream_t s = ctx.stream;
  const int nb = mixed ? choose_nb_grouped(o, v) : choose_nb(o, v, 8, size_t(128) << 20);
  const int64_t NB = ceil_div(v, nb), vp = NB * nb;
  const int64_t o2 = o * o, o3 = o2 * o;

  TriplesSetup T;
  T.o = o;
  T.v = v;
  T.N = N;
  T.nb = nb;
  T.NB = NB;
  T.vp = vp;
  {  // (device time of the whole setup; "phase:" timers enclose other timers)
    TimedScope ts(ctx.timer, "phase:triples_setup", 0.0, 0.0, s);
    T.build(ctx, d_eri, d_t2, d_B, naux, mixed ? Backend::TENSOR : Backend::FP64);
  }
  const DTensor &P = T.P, &Qt = T.Qt, &Rt = T.Rt, &T2p = T.T2p;
  const DevTables &dt = T.dt;
  const size_t kOperand = T.kOperand;

  const int64_t ntrip = v * (v + 1) * (v + 2) / 6;
  DTensor energies({std::max<int64_t>(ntrip, 1)});
  SCESS_CUDA(cudaMemsetAsync(energies.p(), 0, energies.size() * sizeof(double), s));
  // FP64: W in FP64.  MIXED: W in FP32 with rows of (i, j) pairs padded to o2p
  // floats (see pad4), either three buffers the groups store into (nw = 3) or
  // one the groups add into with L2 reductions (nw = 1: zeroed here, cleared
  // again by every energy launch after it has read it)
  const int nw = tune_value("t_wbuf", kTriplesWBuffers) == 3 ? 3 : 1;
  const int64_t o2p = pad4(o2), o3p = o * o2p;
  const size_t wbytes = (size_t)nb * nb * nb * (mixed ? 4 * nw * o3p : 8 * o3);
  DevMem W(wbytes);
  if (mixed && nw == 1) SCESS_CUDA(cudaMemsetAsync(W.as<void>(), 0, wbytes, s));
  const int64_t p1 = o | 1, p2 = (p1 * o) | 1;
  const size_t ysmem = mixed ? (size_t)(4 * o + 2 * o + p2 * o + 3 * p1 * o) * 4
                             : (size_t)(p2 * o + 3 * o2 + 4 * o) * 8;
  if (ysmem > 200 * 1024) throw Error(SCESS_ERR_UNSUPPORTED, "(T): o^3 too large for one CTA");
  if (o > 255) throw Error(SCESS_ERR_UNSUPPORTED, "(T): more than 255 occupied orbitals");
  if (mixed && o > kEnergyMaxO)
    throw Error(SCESS_ERR_UNSUPPORTED, "(T), mixed form: more than 32 occupied orbitals");
  DevMem orbits;
  int norbits = 0;
  if (mixed) {
    SCESS_CUDA(cudaFuncSetAttribute(nw == 1 ? triples_energy_orbit_kernel<1> : triples_energy_orbit_kernel<3>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
    const std::vector<uint32_t> ot = orbit_table(o);
    norbits = (int)ot.size();
    orbits.alloc(ot.size() * sizeof(uint32_t));
    SCESS_CUDA(cudaMemcpyAsync(orbits.as<void>(), ot.data(), ot.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, s));
    ctx.sync();  // (ot is a host vector of this scope)
  } else {
    SCESS_CUDA(cudaFuncSetAttribute(triples_energy_kernel<double, double>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
  }

  // MIXED: the 12 GEMMs of a block triple regroup into three problem sets.
  // Group g has the roles (x, y, z) = (a, b, c), (b, a, c), (c, a, b) and, for
  // each (y_l, z_l), the GEMM
  //   W_g[(u, x_l), (s, t)] =   sum_f P(u,f,x,y) Q(f,s,t,z) + sum_f P(u,f,x,z) Q(f,t,s,y)
  //                           - sum_m t2(m,u,z,x) R(s,t,m,y) - sum_m t2(m,u,y,x) R(t,s,m,z)
  // where u is x's occupied partner (i, j or k for x = a, b, c) and (s, t) the
  // other two occupied indices in order: the P.Q terms of the permutations
  // that put x's pair on the rows and the R.t2 terms whose t2 carries it (four
  // K segments of one accumulation); W = W_0 + W_1 + W_2, each group adding
  // its product into W at its (a, b, c, i, j, k) positions.  The operands are
  // packed once per call into block-grouped FP16 hi/lo rows; the t2 rows are
  // packed negated, and the A side (P, t2) and the B side (Q, R) each share one
  // scale so that all segments carry the same scale product.
  Packed pP, pQ, pQ2, pR, pR2, pTx;
  const int tbn = 256;
  const int tbk = TcEngine::k_block(tbn);
  // 256 x 256 units on cluster pairs of SMs (each SM stages half of B) where
  // the device runs the pair kernel, else one SM per 128 x 256 unit
  const bool tpair = TcEngine::pair_available();
  const int bbox = tpair ? 128 : tbn;  // B rows staged per CTA
  // K block of the t2.R segments (K = o): 32 in the 64-wide kernel when o <= 32
  // (half-filled stages instead of mostly-padding 64-wide ones)
  const int rbk = (tbk == 64 && o <= 32) ? 32 : tbk;
  CUtensorMap mP{}, mQ{}, mQ2{}, mR{}, mR2{}, mTx{};
  DevTables gdt;  // W_g row / column tables
  DevMem Sf;    // (ia|jb) as FP32 for the energy kernel (padded rows)
  DevMem etab;  // eps as FP32 hi + lo (nmo float2), then t1 in FP32
  const int64_t Mg = o * nb, Ng = o2;
  const int64_t Mpq = o * nb * nb, Npq = o2 * nb, Mr = o2 * nb, Nr = o * nb * nb;  // FP64 GEMMs
  if (mixed) {
    TimedScope ts(ctx.timer, "phase:triples_pack", 0.0, 0.0, s);
    TcEngine &tc = ctx.tensor_cores();
    std::vector<TableSpec> pt;
    // P rows r = i + o(x + nb(y + nb(Y + NB X))):  P(i, f, X nb + x, Y nb + y)
    pt.push_back(table({{o, 1}, {nb, o * v}, {nb, o * v * vp}, {NB, o * v * vp * nb}, {NB, o * v * nb}}));
    // Q rows r = j + o(k + o(z + nb Z)):  Q(f, j, k, Z nb + z)
    pt.push_back(table({{o, v}, {o, v * o}, {nb, v * o2}, {NB, v * o2 * nb}}));
    // R rows r = i + o(j + o(x + nb X)):  R(i, j, m, X nb + x)
    pt.push_back(table({{o, 1}, {o, o}, {nb, o3}, {NB, o3 * nb}}));
    // t2 rows r = u + o(x + nb(z + nb(X + NB Z))):  t2(m, u, Z nb + z, X nb + x)
    pt.push_back(table({{o, o}, {nb, o2 * vp}, {nb, o2}, {NB, o2 * vp * nb}, {NB, o2 * nb}}));
    // Q rows in (k, j) order: r = k + o(j + o(z + nb Z))
    pt.push_back(table({{o, v * o}, {o, v}, {nb, v * o2}, {NB, v * o2 * nb}}));
    // R rows in (j, i) order: r = j + o(i + o(x + nb X))
    pt.push_back(table({{o, o}, {o, 1}, {nb, o3}, {NB, o3 * nb}}));
    DevTables pdt;
    pdt.build(ctx, pt);
    DevMem maxw(2 * sizeof(unsigned));
    unsigned *mx = maxw.as<unsigned>();
    SCESS_CUDA(cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned), s));
    tc.maxabs_into(P.p(), pdt.ptr[0], o * vp * vp, dt.ptr[kOperand + 1], v, false, mx);
    tc.maxabs_into(T2p.p(), pdt.ptr[3], o * vp * vp, dt.ptr[kOperand + 7], o, true, mx);
    tc.maxabs_into(Qt.p(), pdt.ptr[1], o2 * vp, dt.ptr[kOperand + 3], v, true, mx + 1);
    tc.maxabs_into(Rt.p(), pdt.ptr[2], o2 * vp, dt.ptr[kOperand + 5], o, false, mx + 1);
    tc.pack_with_max(P.p(), pdt.ptr[0], o * vp * vp, dt.ptr[kOperand + 1], v, false, 128, mx, false, pP);
    tc.pack_with_max(T2p.p(), pdt.ptr[3], o * vp * vp, dt.ptr[kOperand + 7], o, true, 128, mx, true, pTx, rbk);
    tc.pack_with_max(Qt.p(), pdt.ptr[1], o2 * vp, dt.ptr[kOperand + 3], v, true, 128, mx + 1, false, pQ);
    tc.pack_with_max(Qt.p(), pdt.ptr[4], o2 * vp, dt.ptr[kOperand + 3], v, true, 128, mx + 1, false, pQ2);
    tc.pack_with_max(Rt.p(), pdt.ptr[2], o2 * vp, dt.ptr[kOperand + 5], o, false, 128, mx + 1, false, pR, rbk);
    tc.pack_with_max(Rt.p(), pdt.ptr[5], o2 * vp, dt.ptr[kOperand + 5], o, false, 128, mx + 1, false, pR2, rbk);
    ctx.sync();
    // B side (Q, R rows): tiles of tbn columns; 256 halves the A-operand
    // shared-memory traffic per FLOP (SCESS_T_BN=128 selects the narrow tiles).
    // Boxes as wide as the kernel's K block.
    mP = TcEngine::map_of(pP, 128, tbk);
    mQ = TcEngine::map_of(pQ, bbox, tbk);
    mQ2 = TcEngine::map_of(pQ2, bbox, tbk);
    mR = TcEngine::map_of(pR, bbox, rbk);
    mR2 = TcEngine::map_of(pR2, bbox, rbk);
    mTx = TcEngine::map_of(pTx, 128, rbk);
    // Every group writes its (u, s, t) at the triple's (i, j, k), i + o j + o2p k.
    // Rows (u, x_l), columns (s, t): g = 0 (x = a): (u,s,t) = (i,j,k);
    // g = 1 (x = b): (j,i,k); g = 2 (x = c): (k,i,j).  nw = 3: buffer g holds
    // W_g[(y_l nb + z_l) nb + x_l]; nw = 1: W[(a_l nb + b_l) nb + c_l], the
    // (y_l, z_l) strides being the problem offsets cy, cz.
    if (nw == 3)
      gdt.build(ctx, {table({{o, 1}, {nb, o3p}}), table({{o, o}, {o, o2p}}),
                 table({{o, o}, {nb, o3p}}), table({{o, 1}, {o, o2p}}),
                 table({{o, o2p}, {nb, o3p}}), table({{o, 1}, {o, o}})});
    else
      gdt.build(ctx, {table({{o, 1}, {nb, nb * nb * o3p}}), table({{o, o}, {o, o2p}}),
                 table({{o, o}, {nb, nb * o3p}}), table({{o, 1}, {o, o2p}}),
                 table({{o, o2p}, {nb, o3p}}), table({{o, 1}, {o, o}})});
    Sf.alloc((size_t)o2p * v * v * sizeof(float));
    etab.alloc((size_t)N * sizeof(float2) + (size_t)o * v * sizeof(float));
    energy_tables_kernel<<<(unsigned)std::min<int64_t>(ceil_div(N + o * v, 256), 4 * kNumSMs), 256, 0, s>>>(
        d_eps, N, d_t1, o * v, etab.as<float2>(), reinterpret_cast<float *>(etab.as<float2>() + N));
    SCESS_CHECK_LAUNCH();
    to_f32_rows_kernel<<<(unsigned)std::min<int64_t>(ceil_div(o2p * v * v, 256), 16 * kNumSMs), 256, 0, s>>>(
        T.S.p(), v * v, o2, o2p, Sf.as<float>());
    SCESS_CHECK_LAUNCH();
  }
  // (i, j) pairs spread evenly over at most 256 threads
  const unsigned e3threads =
      (unsigned)round_up(ceil_div(o2, ceil_div(o2, 256)), 32);
  double *ws = nullptr;
  if (!mixed) {
    TableGemm probe;
    probe.M = Mpq;
    probe.N = Npq;
    probe.K = v;
    TableGemm probe2;
    probe2.M = Mr;
    probe2.N = Nr;
    probe2.K = o;
    ws = ctx.ensure_workspace(std::max(dgemm_table_workspace(probe), dgemm_table_workspace(probe2)));
  }

  // MIXED: consecutive launches overlap (programmatic dependent launches);
  // SCESS_TUNE t_pdl = 0 serialises them, for comparison
  const bool pdl = tune_value("t_pdl", 1) != 0;
  int64_t blocks_done = 0;
  for (int64_t A = 0; A < NB; A++)
    for (int64_t Bk = 0; Bk <= A; Bk++)
      for (int64_t C = 0; C <= Bk; C++) {
        if ((blocks_done & 15) == 0) ctl.poll();                                   // :123
        const int64_t U[3] = {A, Bk, C};
        if (mixed) {
          TcEngine &tc = ctx.tensor_cores();
          TcProblemSet ps;
          ps.maps[0] = mP;
          ps.maps[1] = mQ;
          ps.maps[2] = mQ2;
          ps.maps[3] = mR;
          ps.maps[4] = mR2;
          ps.maps[5] = mTx;
          ps.nmaps = 6;
          ps.M = Mg;
          ps.N = Ng;
          ps.ny = nb;
          ps.nz = nb;
          ps.ng = 3;
          ps.nseg = 4;
          // TMEM drains per tile.  The FP32 accumulation inside the tensor
          // core truncates, so the error of E_T grows with the products
          // accumulated between drains: measured 1.7e-7 / 4.6e-7 / 1.1e-6
          // relative to FP64 with a drain per 64 / 128 / 256 K.
          ps.kbd = (int)tune_value("t_kbd", kTriplesKbd);
          if (ps.kbd != 1 && ps.kbd != 2 && ps.kbd != 4) ps.kbd = kTriplesKbd;
          ps.bn = tbn;
          ps.bk = tbk;
          ps.pair = tpair;
          // problem offsets of (y_l, z_l): nw = 3, in the group's own buffer;
          // nw = 1, in W with g = 0 (y, z) = (b, c), g = 1 (a, c), g = 2 (a, b)
          for (int g = 0; g < 3; g++) {
            ps.cy[g] = nb * nb * o3p;
            ps.cz[g] = nb * o3p;
          }
          if (nw == 1) {
            ps.cy[0] = nb * o3p;      ps.cz[0] = o3p;
            ps.cy[1] = nb * nb * o3p; ps.cz[1] = o3p;
            ps.cy[2] = nb * nb * o3p; ps.cz[2] = nb * o3p;
          }
          const int kRoles[3][3] = {{0, 1, 2}, {1, 0, 2}, {2, 0, 1}};  // (x, y, z) of group g
          const int64_t rp = o * nb * nb, rq = o2 * nb;                 // block strides of the packs
          TcSegment &s0 = ps.seg[0], &s1 = ps.seg[1], &s2 = ps.seg[2], &s3 = ps.seg[3];
          s0.mapA = 0; s0.mapB = 1; s0.Kpad = pP.Kpad;   // P(u,f,x,y) Q(f,s,t,z)
          s1.mapA = 0; s1.mapB = 2; s1.Kpad = pP.Kpad;   // P(u,f,x,z) Q(f,t,s,y)
          s2.mapA = 5; s2.mapB = 3; s2.Kpad = pTx.Kpad;  // -t2(m,u,z,x) R(s,t,m,y)
          s3.mapA = 5; s3.mapB = 4; s3.Kpad = pTx.Kpad;  // -t2(m,u,y,x) R(t,s,m,z)
          s2.bk = s3.bk = rbk;
          for (int g = 0; g < 3; g++) {
            const int64_t X = U[kRoles[g][0]], Yb = U[kRoles[g][1]], Z = U[kRoles[g][2]];
            ps.cg[g] = nw == 3 ? g * nb * nb * nb * o3p : 0;
            s0.rowA0[g] = rp * (Yb + NB * X); s0.rowAy[g] = o * nb;
            s0.rowB0[g] = rq * Z;             s0.rowBz[g] = o2;
            s1.rowA0[g] = rp * (Z + NB * X);  s1.rowAz[g] = o * nb;
            s1.rowB0[g] = rq * Yb;            s1.rowBy[g] = o2;
            s2.rowA0[g] = rp * (X + NB * Z);  s2.rowAz[g] = o * nb;
            s2.rowB0[g] = rq * Yb;            s2.rowBy[g] = o2;
            s3.rowA0[g] = rp * (X + NB * Yb); s3.rowAy[g] = o * nb;
            s3.rowB0[g] = rq * Z;             s3.rowBz[g] = o2;
          }
          TcOut out;
          out.C = W.as<float>();
          out.fp32 = 1;
          out.rowC = gdt.ptr[0];
          out.colC = gdt.ptr[1];
          for (int g = 0; g < 3; g++) {
            ps.rowC[g] = gdt.ptr[2 * g];
            ps.colC[g] = gdt.ptr[2 * g + 1];
            ps.store_by_column[g] = g > 0;  // i is a column index of groups 1 and 2
            // columns (i, t) with i fastest: quads of i are contiguous and, with
            // o % 4 == 0 (o2p, o3p too), 16-byte aligned
            ps.store_quads[g] = g > 0 && o % 4 == 0;
          }
          out.alpha = 1.0;
          out.beta = nw == 1 ? 1.0 : 0.0;  // nw = 1: W += each group's product (L2 reductions)
          TcEngine::set_scales(out, pP, pQ);
          // In a diagonal block triple a group's problems with y_l < z_l feed no
          // unique triple a >= b >= c: g0 (y, z) = (b, c) when B = C, g1 (a, c)
          // when A = C, g2 (a, b) when A = B.
          ps.tri[0] = Bk == C;
          ps.tri[1] = A == C;
          ps.tri[2] = A == Bk;
          double nprob = 0.0;
          for (int g = 0; g < 3; g++) nprob += ps.tri[g] ? nb * (nb + 1) / 2.0 : (double)nb * nb;
          const double flops = nprob * 2.0 * (double)Mg * Ng * (2.0 * v + 2.0 * o);
          // behind the previous block triple's energy kernel, the launch starts
          // its MMAs while that kernel finishes (W is stored to only after it)
          ps.pdl = pdl && blocks_done > 0;
          tc.gemm_grouped(ps, out, flops, "tc_gemm[triples]");
        } else {
          w_block_fp64(ctx, T, U, W.d(), ws);
        }
        const unsigned nblk = (unsigned)(nb * nb * nb);
        TimedScope ts(ctx.timer, "triples_energy", 0.0,
                      (double)nblk * o3 * (mixed ? (nw == 1 ? 2 : 3) * 4 : 8), s);
        if (mixed) {
          // a programmatic dependent of the grouped GEMM: its CTAs take the SMs
          // that GEMM pairs leave and stage their tables while the last pairs
          // finish; W is read after griddepcontrol.wait
          cudaLaunchConfig_t cfg = {};
          cudaLaunchAttribute at[1];
          at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
          at[0].val.programmaticStreamSerializationAllowed = 1;
          cfg.gridDim = dim3(nblk);
          cfg.blockDim = dim3(e3threads);
          cfg.dynamicSmemBytes = ysmem;
          cfg.stream = s;
          cfg.attrs = at;
          cfg.numAttrs = pdl ? 1 : 0;
          const float *t1f = reinterpret_cast<const float *>(etab.as<float2>() + N);
          SCESS_CUDA(cudaLaunchKernelEx(&cfg, nw == 1 ? triples_energy_orbit_kernel<1> : triples_energy_orbit_kernel<3>,
                                        W.as<float>(), (int64_t)o, (int64_t)v, (int64_t)nb, (int64_t)A,
                                        (int64_t)Bk, (int64_t)C, (const float2 *)etab.as<float2>(), t1f,
                                        (const float *)Sf.as<float>(), (const uint32_t *)orbits.as<uint32_t>(),
                                        norbits, energies.p()));
        } else
          triples_energy_kernel<double, double><<<nblk, 256, ysmem, s>>>(
              W.d(), o, v, nb, A, Bk, C, d_eps, d_t1, T.S.p(), energies.p());
        SCESS_CHECK_LAUNCH();
        blocks_done++;
      }
  sum_energies_kernel<<<1, 1024, 0, s>>>(ntrip, energies.p(), ctx.dscalars);
  SCESS_CHECK_LAUNCH();
  SCESS_CUDA(cudaMemcpyAsync(ctx.hscalars, ctx.dscalars, sizeof(double), cudaMemcpyDeviceToHost, s));
  ctx.sync();
  if (mixed) ctx.tensor_cores().check_error();
  if (stats) {
    stats->nb = nb;
    stats->block_triples = blocks_done;
  }
  return ctx.hscalars[0];
}

double rccsd_triples_vjp(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t o,
                         const double *d_eps, const double *d_t1, const double *d_t2, double gE,
                         const Control &ctl, double *d_gt1, double *d_gt2, double *d_geri,
                         bool mixed) {
  const int64_t v = nmo - o, N = nmo;
  cudaStream_t s = ctx.stream;
  const int nb = choose_nb(o, v, 8, size_t(64) << 20);  // W and G, nb^3 o^3 FP64 each
  const int64_t NB = ceil_div(v, nb), vp = NB * nb;
  const int64_t o2 = o * o, o3 = o2 * o, N2 = N * N, N3 = N2 * N;
  TriplesSetup T;
  T.o = o;
  T.v = v;
  T.N = N;
  T.nb = nb;
  T.NB = NB;
  T.vp = vp;
  T.build(ctx, d_eri, d_t2);
  const bool integrals = d_geri != nullptr;
  DTensor gP, gRt;
  if (integrals) {
    gP = DTensor({o, v, vp, vp});
    gRt = DTensor({o, o, o, vp});
    SCESS_CUDA(cudaMemsetAsync(gP.p(), 0, gP.size() * sizeof(double), s));
    SCESS_CUDA(cudaMemsetAsync(gRt.p(), 0, gRt.size() * sizeof(double), s));
  }
  DTensor gQt({v, o, o, vp}), gT2p({o, o, vp, vp}), gS({o, o, v, v});
  SCESS_CUDA(cudaMemsetAsync(gQt.p(), 0, gQt.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(gT2p.p(), 0, gT2p.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(gS.p(), 0, gS.size() * sizeof(double), s));
  const int64_t ntrip = v * (v + 1) * (v + 2) / 6;
  DTensor energies({std::max<int64_t>(ntrip, 1)});
  SCESS_CUDA(cudaMemsetAsync(energies.p(), 0, energies.size() * sizeof(double), s));
  DevMem W((size_t)o3 * nb * nb * nb * 8), G((size_t)o3 * nb * nb * nb * 8);
  const int64_t p1 = o | 1, p2 = (p1 * o) | 1;
  const size_t gsmem = (size_t)(p2 * o + 5 * o2 + 7 * o) * 8;
  if (gsmem > 200 * 1024) throw Error(SCESS_ERR_UNSUPPORTED, "(T) gradient: o^3 too large for one CTA");
  SCESS_CUDA(cudaFuncSetAttribute(triples_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)gsmem));
  int64_t need = 0;
  {
    const int64_t shapes[6][3] = {{T.Mpq(), T.Npq(), v}, {T.Mr(), T.Nr(), o}, {T.Mpq(), v, T.Npq()},
                                  {T.Npq(), v, T.Mpq()}, {T.Mr(), o, T.Nr()}, {T.Nr(), o, T.Mr()}};
    for (auto &sh : shapes) {
      TableGemm probe;
      probe.M = sh[0];
      probe.N = sh[1];
      probe.K = sh[2];
      need = std::max(need, dgemm_table_workspace(probe));
    }
  }
  double *ws = ctx.ensure_workspace(need);
  int64_t blocks_done = 0;
  for (int64_t A = 0; A < NB; A++)
    for (int64_t Bk = 0; Bk <= A; Bk++)
      for (int64_t C = 0; C <= Bk; C++) {
        if ((blocks_done & 15) == 0) ctl.poll();
        const int64_t U[3] = {A, Bk, C};
        w_block_fp64(ctx, T, U, W.d(), ws, mixed);
        {
          TimedScope ts(ctx.timer, "triples_grad", 0.0, 0.0, s);
          triples_grad_kernel<<<(unsigned)(nb * nb * nb), 256, gsmem, s>>>(
              W.d(), G.d(), o, v, nb, A, Bk, C, d_eps, d_t1, T.S.p(), gE, energies.p(), d_gt1,
              gS.p());
          SCESS_CHECK_LAUNCH();
        }
        g_block_fp64(ctx, T, U, G.d(), integrals ? gP.p() : nullptr, gQt.p(),
                     integrals ? gRt.p() : nullptr, gT2p.p(), integrals, ws, mixed);
        blocks_done++;
      }
  sum_energies_kernel<<<1, 1024, 0, s>>>(ntrip, energies.p(), ctx.dscalars);
  SCESS_CHECK_LAUNCH();
  SCESS_CUDA(cudaMemcpyAsync(ctx.hscalars, ctx.dscalars, sizeof(double), cudaMemcpyDeviceToHost, s));
  if (mixed) ctx.tensor_cores().check_error();

  // back through the repacks (RCCSD_T.cpp:30-56) into t2 and eri
  const TV g_t2 = cm(d_gt2, {o, o, v, v});
  TV q = gQt.v;  // Q(f,j,k,c) = t2(k,j,c,f)
  q.ext[3] = v;
  permute(ctx, "fjkc->kjcf", 1.0, q, 1.0, g_t2);
  TV t = gT2p.v;
  t.ext[2] = v;
  t.ext[3] = v;
  permute(ctx, "mkbc->mkbc", 1.0, t, 1.0, g_t2);
  if (integrals) {
    auto view = [&](int64_t off, std::initializer_list<int64_t> ext) {
      TV e;
      e.p = d_geri + off;
      e.nd = 4;
      int k = 0;
      for (int64_t x : ext) e.ext[k++] = x;
      const int64_t st[4] = {1, N, N2, N3};
      std::memcpy(e.str, st, sizeof(st));
      return e;
    };
    TV pv = gP.v;  // P(i,f,a,b) = eri(i, o+b, o+a, o+f)
    pv.ext[2] = v;
    pv.ext[3] = v;
    permute(ctx, "ifab->ibaf", 1.0, pv, 1.0, view(o * N + o * N2 + o * N3, {o, v, v, v}));
    TV rv = gRt.v;  // R(i,j,m,a) = eri(i, m, o+a, j)
    rv.ext[3] = v;
    permute(ctx, "ijma->imaj", 1.0, rv, 1.0, view(o * N2, {o, o, v, o}));
    // S(i,j,a,b) = eri(i, j, o+a, o+b)
    permute(ctx, "ijab->ijab", 1.0, gS.v, 1.0, view(o * N2 + o * N3, {o, o, v, v}));
  }
  ctx.sync();
  return ctx.hscalars[0];
}

}  // namespace scess
