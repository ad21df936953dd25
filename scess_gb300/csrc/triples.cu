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
// FP64 energy arithmetic.  MIXED form: the operands are packed once per call
// into BF16 hi/lo rows grouped by block, the GEMMs run on tcgen05 tensor
// cores into an FP32 W, and the energy kernel works in FP32 per element with
// FP64 accumulation per triple.
#include <cmath>
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
__device__ __forceinline__ float div_fast(float x, float y) { return __fdividef(x, y); }
__device__ __forceinline__ double div_fast(double x, double y) { return x / y; }

// One CTA per local triple (a_l, b_l, c_l) of the block triple (A, B, C).
// Shared memory: Y (o^3) then Sbc, Sac, Sab (o^2 each) then t1 columns and the
// occupied orbital energies (o each), all in the arithmetic type CT.
template <typename WT, typename CT>
__global__ void __launch_bounds__(256) triples_energy_kernel(
    const WT *__restrict__ W, int64_t o, int64_t v, int64_t nb, int64_t A, int64_t Bk, int64_t C,
    const double *__restrict__ eps, const double *__restrict__ t1, const double *__restrict__ eri,
    int64_t N, double *__restrict__ energies) {
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
  // S(i,j,a,b) = (ia|jb) = eri(i, j, o+a, o+b)
  const int64_t N2 = N * N, N3 = N2 * N;
  for (int e = threadIdx.x; e < o2; e += blockDim.x) {
    const int i = e % oo, j = e / oo;
    Sbc[e] = (CT)eri[i + N * j + (o + b) * N2 + (o + c) * N3];
    Sac[e] = (CT)eri[i + N * j + (o + a) * N2 + (o + c) * N3];
    Sab[e] = (CT)eri[i + N * j + (o + a) * N2 + (o + b) * N3];
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

// Offset table over a list of (extent, stride) dims, first fastest.
std::vector<int64_t> table(std::initializer_list<std::pair<int64_t, int64_t>> dims) {
  int64_t n = 1;
  for (auto &d : dims) n *= d.first;
  std::vector<int64_t> t((size_t)n);
  for (int64_t e = 0; e < n; e++) {
    int64_t r = e, off = 0;
    for (auto &d : dims) {
      off += (r % d.first) * d.second;
      r /= d.first;
    }
    t[(size_t)e] = off;
  }
  return t;
}

struct DevTables {
  DevMem mem;
  std::vector<const int64_t *> ptr;
  void build(const std::vector<std::vector<int64_t>> &ts) {
    size_t tot = 0;
    for (auto &t : ts) tot += t.size();
    mem.alloc(std::max<size_t>(tot, 1) * sizeof(int64_t));
    size_t off = 0;
    ptr.clear();
    for (auto &t : ts) {
      ptr.push_back(mem.as<int64_t>() + off);
      SCESS_CUDA(cudaMemcpy(mem.as<int64_t>() + off, t.data(), t.size() * sizeof(int64_t),
                            cudaMemcpyHostToDevice));
      off += t.size();
    }
  }
};

// The six simultaneous permutations of Symmetrise, as position maps: the raw
// term w^{u[p0] u[p1] u[p2]}_{w[p0] w[p1] w[p2]} feeds W^{abc}_{ijk}.
const int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

int choose_nb(int64_t o, int64_t v, size_t welem_bytes, size_t budget) {
  const double o3 = (double)o * o * o;
  int nb = (int)std::floor(std::cbrt((double)budget / (welem_bytes * o3)));
  nb = std::max(1, std::min<int>(nb, (int)v));
  // balance the blocks over v
  const int64_t nblk = ceil_div(v, nb);
  nb = (int)ceil_div(v, nblk);
  return nb;
}

}  // namespace

double rccsd_triples(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t o, const double *d_eps,
                     const double *d_t1, const double *d_t2, bool mixed, const Control &ctl,
                     TriplesStats *stats) {
  const int64_t v = nmo - o, N = nmo;
  cudaStream_t s = ctx.stream;
  const int nb = mixed ? choose_nb(o, v, 4, size_t(64) << 20) : choose_nb(o, v, 8, size_t(128) << 20);
  const int64_t NB = ceil_div(v, nb), vp = NB * nb;
  const int64_t o2 = o * o, o3 = o2 * o;
  const int64_t N2 = N * N, N3 = N2 * N;

  // Zero-padded FP64 repacks (RCCSD_T.cpp:30-56), virtual indices padded to vp.
  DTensor P({o, v, vp, vp});   // P(i,f,a,b) = (ia|bf) = eri(i, o+b, o+a, o+f)
  DTensor Qt({v, o, o, vp});   // Q(f,j,k,c) = t2(k,j,c,f)
  DTensor Rt({o, o, o, vp});   // R(i,j,m,a) = (ia|mj) = eri(i, m, o+a, j)
  DTensor T2p({o, o, vp, vp}); // t2(m,k,b,c)
  SCESS_CUDA(cudaMemsetAsync(P.p(), 0, P.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(Qt.p(), 0, Qt.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(Rt.p(), 0, Rt.size() * sizeof(double), s));
  SCESS_CUDA(cudaMemsetAsync(T2p.p(), 0, T2p.size() * sizeof(double), s));
  {
    TV e;  // (i, b, a, f) -> eri(i, o+b, o+a, o+f)
    e.p = const_cast<double *>(d_eri) + o * N + o * N2 + o * N3;
    e.nd = 4;
    int64_t ee[4] = {o, v, v, v}, es[4] = {1, N, N2, N3};
    std::memcpy(e.ext, ee, sizeof(ee));
    std::memcpy(e.str, es, sizeof(es));
    TV Pv = P.v;
    Pv.ext[2] = v;
    Pv.ext[3] = v;
    permute(ctx, "ibaf->ifab", 1.0, e, 0.0, Pv);
    TV r;  // (i, m, a, j) -> eri(i, m, o+a, j)
    r.p = const_cast<double *>(d_eri) + o * N2;
    r.nd = 4;
    int64_t re[4] = {o, o, v, o}, rs[4] = {1, N, N2, N3};
    std::memcpy(r.ext, re, sizeof(re));
    std::memcpy(r.str, rs, sizeof(rs));
    TV Rv = Rt.v;
    Rv.ext[3] = v;
    permute(ctx, "imaj->ijma", 1.0, r, 0.0, Rv);
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
  auto q_swapped = [](const int *pi) { return pi[2] == 0; };
  auto r_swapped = [](const int *pi) { return pi[1] == 0; };
  std::vector<std::vector<int64_t>> ts;
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
  const size_t kOperand = ts.size();
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
  DevTables dt;
  dt.build(ts);

  const int64_t ntrip = v * (v + 1) * (v + 2) / 6;
  DTensor energies({std::max<int64_t>(ntrip, 1)});
  SCESS_CUDA(cudaMemsetAsync(energies.p(), 0, energies.size() * sizeof(double), s));
  const size_t wbytes = (size_t)o3 * nb * nb * nb * (mixed ? 4 : 8);
  DevMem W(wbytes);
  const int64_t p1 = o | 1, p2 = (p1 * o) | 1;
  const size_t ysmem = (size_t)(p2 * o + 3 * o2 + 4 * o) * (mixed ? 4 : 8);
  if (ysmem > 200 * 1024) throw Error(SCESS_ERR_UNSUPPORTED, "(T): o^3 too large for one CTA");
  if (mixed) {
    SCESS_CUDA(cudaFuncSetAttribute(triples_energy_kernel<float, float>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
  } else {
    SCESS_CUDA(cudaFuncSetAttribute(triples_energy_kernel<double, double>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
  }

  // MIXED: pack the operands once into block-grouped BF16 hi/lo rows.
  Packed pP, pQ, pQ2, pR, pR2, pT;
  CUtensorMap mP{}, mQ{}, mQ2{}, mR{}, mR2{}, mT{};
  const int64_t Mpq = o * nb * nb, Npq = o2 * nb, Mr = o2 * nb, Nr = o * nb * nb;
  if (mixed) {
    TcEngine &tc = ctx.tensor_cores();
    std::vector<std::vector<int64_t>> pt;
    // P rows r = i + o(x + nb(y + nb(Y + NB X)))
    pt.push_back(table({{o, 1}, {nb, o * v}, {nb, o * v * vp}, {NB, o * v * vp * nb}, {NB, o * v * nb}}));
    // Q rows r = j + o(k + o(z + nb Z))
    pt.push_back(table({{o, v}, {o, v * o}, {nb, v * o2}, {NB, v * o2 * nb}}));
    // R rows r = i + o(j + o(x + nb X))
    pt.push_back(table({{o, 1}, {o, o}, {nb, o3}, {NB, o3 * nb}}));
    // t2 rows r = k + o(y + nb(z + nb(Z + NB Y)))
    pt.push_back(table({{o, o}, {nb, o2}, {nb, o2 * vp}, {NB, o2 * vp * nb}, {NB, o2 * nb}}));
    // Q rows in (k, j) order: r = k + o(j + o(z + nb Z))
    pt.push_back(table({{o, v * o}, {o, v}, {nb, v * o2}, {NB, v * o2 * nb}}));
    // R rows in (j, i) order: r = j + o(i + o(x + nb X))
    pt.push_back(table({{o, o}, {o, 1}, {nb, o3}, {NB, o3 * nb}}));
    DevTables pdt;
    pdt.build(pt);
    tc.pack(P.p(), pdt.ptr[0], o * vp * vp, dt.ptr[kOperand + 1], v, false, 128, pP);
    tc.pack(Qt.p(), pdt.ptr[1], o2 * vp, dt.ptr[kOperand + 3], v, true, 128, pQ);
    tc.pack(Qt.p(), pdt.ptr[4], o2 * vp, dt.ptr[kOperand + 3], v, true, 128, pQ2);
    tc.pack(Rt.p(), pdt.ptr[2], o2 * vp, dt.ptr[kOperand + 5], o, false, 128, pR);
    tc.pack(Rt.p(), pdt.ptr[5], o2 * vp, dt.ptr[kOperand + 5], o, false, 128, pR2);
    tc.pack(T2p.p(), pdt.ptr[3], o * vp * vp, dt.ptr[kOperand + 7], o, true, 128, pT);
    ctx.sync();
    mP = TcEngine::map_of(pP, 128);
    mQ = TcEngine::map_of(pQ, TcEngine::tile_n(Npq));
    mQ2 = TcEngine::map_of(pQ2, TcEngine::tile_n(Npq));
    mR = TcEngine::map_of(pR, 128);
    mR2 = TcEngine::map_of(pR2, 128);
    mT = TcEngine::map_of(pT, TcEngine::tile_n(Nr));
  }
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

  int64_t blocks_done = 0;
  for (int64_t A = 0; A < NB; A++)
    for (int64_t Bk = 0; Bk <= A; Bk++)
      for (int64_t C = 0; C <= Bk; C++) {
        if ((blocks_done & 15) == 0) ctl.poll();                                   // :123
        const int64_t U[3] = {A, Bk, C};
        for (int p = 0; p < 6; p++) {
          const int *pi = kPerm[p];
          const int64_t X = U[pi[0]], Yb = U[pi[1]], Z = U[pi[2]];
          const int64_t *rowPQ = dt.ptr[4 * p + 0], *colPQ = dt.ptr[4 * p + 1];
          const int64_t *rowR = dt.ptr[4 * p + 2], *colR = dt.ptr[4 * p + 3];
          if (mixed) {
            TcEngine &tc = ctx.tensor_cores();
            TcOut out;
            out.C = W.as<float>();
            out.fp32 = 1;
            out.rowC = rowPQ;
            out.colC = colPQ;
            out.alpha = 1.0;
            out.beta = p == 0 ? 0.0 : 1.0;
            const bool qs = q_swapped(pi), rs = r_swapped(pi);
            // Lane side (GEMM rows) = the operand whose first index is W's i:
            // P rows (i',x,y) when i' is i, else the Q columns (j'/k' first).
            const Packed &pq = qs ? pQ2 : pQ;
            const CUtensorMap &mq = qs ? mQ2 : mQ;
            if (pi[0] == 0) {
              TcEngine::set_scales(out, pP, pq);
              tc.gemm_maps(mP, mq, pP.Kpad, v, Mpq * (X * NB + Yb), Mpq, Npq * Z, Npq, out);
            } else {
              out.rowC = colPQ;
              out.colC = rowPQ;
              TcEngine::set_scales(out, pq, pP);
              tc.gemm_maps(mq, mP, pP.Kpad, v, Npq * Z, Npq, Mpq * (X * NB + Yb), Mpq, out);
            }
            out.alpha = -1.0;
            out.beta = 1.0;
            const Packed &pr = rs ? pR2 : pR;
            const CUtensorMap &mr = rs ? mR2 : mR;
            if (pi[2] != 0) {  // R rows (i',j',x) / (j',i',x) start with W's i
              out.rowC = rowR;
              out.colC = colR;
              TcEngine::set_scales(out, pr, pT);
              tc.gemm_maps(mr, mT, pR.Kpad, o, Mr * X, Mr, Nr * (Yb * NB + Z), Nr, out);
            } else {           // k' is W's i: t2 rows (k',y,z) on the lane side
              out.rowC = colR;
              out.colC = rowR;
              TcEngine::set_scales(out, pT, pr);
              tc.gemm_maps(mT, mr, pR.Kpad, o, Nr * (Yb * NB + Z), Nr, Mr * X, Mr, out);
            }
          } else {
            TableGemm g;
            g.A = P.p();
            g.B = Qt.p();
            g.C = W.d();
            g.rowA = dt.ptr[kOperand + 0];
            g.kA = dt.ptr[kOperand + 1];
            g.colB = dt.ptr[kOperand + (q_swapped(pi) ? 8 : 2)];
            g.kB = dt.ptr[kOperand + 3];
            g.rowC = rowPQ;
            g.colC = colPQ;
            g.baseA = o * v * (X * nb) + o * v * vp * (Yb * nb);
            g.baseB = v * o2 * (Z * nb);
            g.M = Mpq;
            g.N = Npq;
            g.K = v;
            g.alpha = 1.0;
            g.beta = p == 0 ? 0.0 : 1.0;
            g.aUnitM = 1;
            g.bUnitN = 0;
            {
              TimedScope ts(ctx.timer, "dgemm_table", 2.0 * g.M * g.N * g.K, 0.0, s);
              dgemm_table(g, ws, s);
            }
            TableGemm h;
            h.A = Rt.p();
            h.B = T2p.p();
            h.C = W.d();
            h.rowA = dt.ptr[kOperand + (r_swapped(pi) ? 9 : 4)];
            h.kA = dt.ptr[kOperand + 5];
            h.colB = dt.ptr[kOperand + 6];
            h.kB = dt.ptr[kOperand + 7];
            h.rowC = rowR;
            h.colC = colR;
            h.baseA = o3 * (X * nb);
            h.baseB = o2 * (Yb * nb) + o2 * vp * (Z * nb);
            h.M = Mr;
            h.N = Nr;
            h.K = o;
            h.alpha = -1.0;
            h.beta = 1.0;
            h.aUnitM = r_swapped(pi) ? 0 : 1;
            h.bUnitN = 0;
            TimedScope ts(ctx.timer, "dgemm_table", 2.0 * h.M * h.N * h.K, 0.0, s);
            dgemm_table(h, ws, s);
          }
        }
        const unsigned nblk = (unsigned)(nb * nb * nb);
        TimedScope ts(ctx.timer, "triples_energy", 0.0, (double)nblk * o3 * (mixed ? 4 : 8), s);
        if (mixed)
          triples_energy_kernel<float, float><<<nblk, 256, ysmem, s>>>(
              W.as<float>(), o, v, nb, A, Bk, C, d_eps, d_t1, d_eri, N, energies.p());
        else
          triples_energy_kernel<double, double><<<nblk, 256, ysmem, s>>>(
              W.d(), o, v, nb, A, Bk, C, d_eps, d_t1, d_eri, N, energies.p());
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

}  // namespace scess
