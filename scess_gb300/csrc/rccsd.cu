// Closed-shell CCSD: integral block views, residual op list, solver loop with DIIS.
//
// Follows SCESS src/Quantum/CC/RCCSD.cpp:
//   MakeIntegralBlocks :47-72 -> RccsdBlocks::build (strided views, no copies)
//   UpdateAmplitudes   :101-237 -> rccsd_residual + divide_denominators
//   AmplitudeDIIS      :240-279 -> device vectors + host Gram/full-pivot LU
//   SolveRCCSD_DIIS    :295-394 -> rccsd_solve
#include <cfloat>
#include <cmath>
#include <cstring>

#include "gemm_tc.h"
#include "rccsd.h"

namespace scess {

namespace {

TV view(double *base, int64_t off, std::initializer_list<int64_t> ext,
        std::initializer_list<int64_t> str) {
  TV t;
  t.p = base + off;
  t.nd = (int)ext.size();
  int d = 0;
  for (int64_t e : ext) t.ext[d++] = e;
  d = 0;
  for (int64_t s : str) t.str[d++] = s;
  return t;
}

}  // namespace

void RccsdBlocks::build(Ctx &ctx, const double *d_eri, int64_t nmo, int64_t nocc) {
  o = nocc;
  v = nmo - nocc;
  N = nmo;
  double *e = const_cast<double *>(d_eri);
  const int64_t N1 = 1, N2 = N, N3 = N * N, N4 = N * N * N;  // strides of p, q, r, s
  // eri(p,q,r,s) = <pq|rs> at p + N q + N^2 r + N^3 s
  // ovov(k,c,l,d) = (kc|ld) = <kl|cd> = eri(k, l, o+c, o+d)                       :55
  ovov = view(e, o * N3 + o * N4, {o, v, o, v}, {N1, N3, N2, N4});
  // oovv(k,i,a,c) = (ki|ac) = <ka|ic> = eri(k, o+a, i, o+c)                       :57
  oovv = view(e, o * N2 + o * N4, {o, o, v, v}, {N1, N3, N2, N4});
  // ovvo(k,c,a,i) = (kc|ai) = <ka|ci> = eri(k, o+a, o+c, i)                       :59
  ovvo = view(e, o * N2 + o * N3, {o, v, v, o}, {N1, N3, N2, N4});
  // ovvv(k,d,a,c) = (kd|ac) = <ka|dc> = eri(k, o+a, o+d, o+c)                     :61
  ovvv = view(e, o * N2 + o * N3 + o * N4, {o, v, v, v}, {N1, N3, N2, N4});
  // ovoo(l,c,k,i) = (lc|ki) = <lk|ci> = eri(l, k, o+c, i)                         :63
  ovoo = view(e, o * N3, {o, v, o, o}, {N1, N3, N2, N4});
  // oooo_phys(k,l,i,j) = <kl|ij>                                                    :64
  oooo = view(e, 0, {o, o, o, o}, {N1, N2, N3, N4});
  // vvvv_phys(a,b,c,d) = <ab|cd>                                                    :65
  vvvv = view(e, o * (N1 + N2 + N3 + N4), {v, v, v, v}, {N1, N2, N3, N4});
  // oovv_phys(i,j,a,b) = <ij|ab>                                                    :66
  oovv_phys = view(e, o * N3 + o * N4, {o, o, v, v}, {N1, N2, N3, N4});
  build_l(ctx);
}

void RccsdBlocks::build_df(Ctx &ctx, const double *d_B, int64_t naux, int64_t nmo, int64_t nocc,
                           Backend be) {
  o = nocc;
  v = nmo - nocc;
  N = nmo;
  regions.clear();
  regions.reserve(7);
  // <pq|rs> = (pr|qs) = sum_Q B(Q,p,r) B(Q,q,s) over the index ranges of one
  // region, stored (p, q, r, s) column-major
  auto region = [&](int64_t p0, int64_t np, int64_t q0, int64_t nq, int64_t r0, int64_t nr,
                    int64_t s0, int64_t ns) -> double * {
    auto bview = [&](int64_t a0, int64_t na, int64_t b0, int64_t nb) {
      TV t;
      t.p = const_cast<double *>(d_B) + naux * a0 + naux * N * b0;
      t.nd = 3;
      const int64_t e3[3] = {naux, na, nb}, s3[3] = {1, naux, naux * N};
      std::memcpy(t.ext, e3, sizeof(e3));
      std::memcpy(t.str, s3, sizeof(s3));
      return t;
    };
    regions.emplace_back(DTensor({np, nq, nr, ns}));
    einsum(ctx, "Qpr,Qqs->pqrs", 1.0, bview(p0, np, r0, nr), bview(q0, nq, s0, ns), 0.0,
           regions.back().v, be);
    return regions.back().p();
  };
  auto tv = [](double *p, std::initializer_list<int64_t> ext, std::initializer_list<int64_t> str) {
    TV t;
    t.p = p;
    t.nd = (int)ext.size();
    int d = 0;
    for (int64_t e : ext) t.ext[d++] = e;
    d = 0;
    for (int64_t x : str) t.str[d++] = x;
    return t;
  };
  const int64_t o2 = o * o, ov = o * v;
  // <kl|cd>: ovov(k,c,l,d) and oovv_phys(i,j,a,b)                               :55, :66
  double *r_oovv = region(0, o, 0, o, o, v, o, v);
  ovov = tv(r_oovv, {o, v, o, v}, {1, o2, o, o2 * v});
  oovv_phys = tv(r_oovv, {o, o, v, v}, {1, o, o2, o2 * v});
  // <ka|ic>: oovv(k,i,a,c)                                                        :57
  oovv = tv(region(0, o, o, v, 0, o, o, v), {o, o, v, v}, {1, ov, o, o2 * v});
  // <ka|ci>: ovvo(k,c,a,i)                                                        :59
  ovvo = tv(region(0, o, o, v, o, v, 0, o), {o, v, v, o}, {1, ov, o, ov * v});
  // <ka|dc>: ovvv(k,d,a,c)                                                        :61
  ovvv = tv(region(0, o, o, v, o, v, o, v), {o, v, v, v}, {1, ov, o, ov * v});
  // <lk|ci>: ovoo(l,c,k,i)                                                        :63
  ovoo = tv(region(0, o, 0, o, o, v, 0, o), {o, v, o, o}, {1, o2, o, o2 * v});
  // <kl|ij>, <ab|cd>                                                           :64-65
  oooo = tv(region(0, o, 0, o, 0, o, 0, o), {o, o, o, o}, {1, o, o2, o2 * o});
  vvvv = tv(region(o, v, o, v, o, v, o, v), {v, v, v, v}, {1, v, v * v, v * v * v});
  build_l(ctx);
}

const TV &RccsdBlocks::l_ovvv(Ctx &ctx) const {
  if (!L_ovvv.p()) {
    L_ovvv = DTensor({o, v, v, v});
    permute(ctx, "kdac->kdac", 2.0, ovvv, 0.0, L_ovvv.v);
    permute(ctx, "kcad->kdac", -1.0, ovvv, 1.0, L_ovvv.v);
  }
  return L_ovvv.v;
}

const TV &RccsdBlocks::l_ovoo(Ctx &ctx) const {
  if (!L_ovoo.p()) {
    L_ovoo = DTensor({o, v, o, o});
    permute(ctx, "lcki->lcki", 2.0, ovoo, 0.0, L_ovoo.v);
    permute(ctx, "kcli->lcki", -1.0, ovoo, 1.0, L_ovoo.v);
  }
  return L_ovoo.v;
}

void RccsdBlocks::build_l(Ctx &ctx) {
  // L_oovv = 2 <ij|ab> - <ij|ba>                                                   :68-69
  L_oovv = DTensor({o, o, v, v});
  permute(ctx, "ijab->ijab", 2.0, oovv_phys, 0.0, L_oovv.v);
  permute(ctx, "ijba->ijab", -1.0, oovv_phys, 1.0, L_oovv.v);
  // L_ovov = 2 (kc|ld) - (kd|lc)                                                   :70
  L_ovov = DTensor({o, v, o, v});
  permute(ctx, "kcld->kcld", 2.0, ovov, 0.0, L_ovov.v);
  permute(ctx, "kdlc->kcld", -1.0, ovov, 1.0, L_ovov.v);
}

void ladder_pm(Ctx &ctx, const RccsdBlocks &B, const TV &tau, double *R2, Backend be) {
  const int64_t o = B.o, v = B.v;
  cudaStream_t s = ctx.stream;
  if (!B.ladder) {
    auto L = std::make_unique<LadderPM>();
    L->nuo = o * (o + 1) / 2;
    L->nso = o * (o - 1) / 2;
    L->nuv = v * (v + 1) / 2;
    L->nsv = v * (v - 1) / 2;
    std::vector<int2> pr;
    auto add = [&](int64_t n, bool strict) {
      for (int64_t q = 0; q < n; q++)
        for (int64_t p = 0; p < (strict ? q : q + 1); p++) pr.push_back(make_int2((int)p, (int)q));
    };
    add(o, false);
    add(o, true);
    add(v, false);
    add(v, true);
    L->pairs.alloc(std::max<size_t>(pr.size(), 1) * sizeof(int2));
    SCESS_CUDA(cudaMemcpyAsync(L->pairs.as<void>(), pr.data(), pr.size() * sizeof(int2),
                               cudaMemcpyHostToDevice, s));
    L->pu_o = L->pairs.as<int2>();
    L->ps_o = L->pu_o + L->nuo;
    L->pu_v = L->ps_o + L->nso;
    L->ps_v = L->pu_v + L->nuv;
    L->Vp = DTensor({L->nuv, L->nuv});
    L->Vm = DTensor({std::max<int64_t>(L->nsv, 1), std::max<int64_t>(L->nsv, 1)});
    ladder_vpm(B.vvvv.p, B.vvvv.str[0], B.vvvv.str[1], B.vvvv.str[2], B.vvvv.str[3], L->pu_v,
               L->nuv, L->ps_v, L->nsv, L->Vp.p(), L->Vm.p(), s);
    L->Tp = DTensor({L->nuo, L->nuv});
    L->Tm = DTensor({std::max<int64_t>(L->nso, 1), std::max<int64_t>(L->nsv, 1)});
    L->Sp = DTensor({L->nuo, L->nuv});
    L->Sm = DTensor({std::max<int64_t>(L->nso, 1), std::max<int64_t>(L->nsv, 1)});
    ctx.sync();  // (pr is a host vector of this scope)
    B.ladder = std::move(L);
  }
  LadderPM &L = *B.ladder;
  ladder_tpm(o, v, tau.p, L.pu_o, L.nuo, L.ps_o, L.nso, L.pu_v, L.nuv, L.ps_v, L.nsv, L.Tp.p(),
             L.Tm.p(), s);
  // S+(y, x) = sum_k T+(y, k) V+(x, k); the same for the strict pairs
  einsum(ctx, "yk,xk->yx", 1.0, cm(L.Tp.p(), {L.nuo, L.nuv}), cm(L.Vp.p(), {L.nuv, L.nuv}), 0.0,
         cm(L.Sp.p(), {L.nuo, L.nuv}), be, false, true);
  if (L.nso > 0 && L.nsv > 0)
    einsum(ctx, "yk,xk->yx", 1.0, cm(L.Tm.p(), {L.nso, L.nsv}), cm(L.Vm.p(), {L.nsv, L.nsv}), 0.0,
           cm(L.Sm.p(), {L.nso, L.nsv}), be, false, true);
  else
    SCESS_CUDA(cudaMemsetAsync(L.Sm.p(), 0, L.Sm.size() * sizeof(double), s));
  ladder_unpack(o, v, L.Sp.p(), L.Sm.p(), R2, s);
}

void RccsdWork::alloc(int64_t o, int64_t v, bool direct_vvvv) {
  tau = DTensor({o, o, v, v});
  Foo = DTensor({o, o});
  Fvv = DTensor({v, v});
  Fov = DTensor({o, v});
  Fovt1 = DTensor({o, o});
  Loo = DTensor({o, o});
  Lvv = DTensor({v, v});
  X = DTensor({o, o, v, v});
  tmp_abic = DTensor({v, v, o, v});
  tmp_kibj = DTensor({o, o, v, o});
  tmp_akij = DTensor({v, o, o, o});
  Woooo = DTensor({o, o, o, o});
  Wvoov = DTensor({v, o, o, v});
  Wvovo = DTensor({v, o, v, o});
  tmp_lkci = DTensor({o, o, v, o});
  tmp_lcki = DTensor({o, v, o, o});
  Yd = DTensor({o, v, o, o});
  if (direct_vvvv) Wvvvv = DTensor({v, v, v, v});
}

// Shared max|x| of tensors a residual packs several times (TcEngine max
// hints), for the calls that run on the tensor cores; cleared on scope exit.
struct MaxHints {
  TcEngine *tc = nullptr;
  MaxHints(Ctx &ctx, Backend be) {
    if (be != Backend::FP64) tc = &ctx.tensor_cores();
  }
  void add(const double *p, int64_t n) {
    if (tc) tc->add_max_hint(p, n);
  }
  ~MaxHints() {
    if (tc) tc->clear_max_hints();
  }
  MaxHints(const MaxHints &) = delete;
  MaxHints &operator=(const MaxHints &) = delete;
};

void rccsd_residual(Ctx &ctx, const RccsdBlocks &B, const double *amp, const double *t2driver,
                    Backend be, RccsdWork &w, double *R, ResidualList list) {
  const int64_t o = B.o, v = B.v;
  const bool literal = list == ResidualList::AUTO ? be == Backend::FP64 : list == ResidualList::LITERAL;
  cudaStream_t s = ctx.stream;
  double *a = const_cast<double *>(amp);
  const TV t1 = cm(a, {o, v});
  const TV t2 = cm(a + o * v, {o, o, v, v});
  const TV R1 = cm(R, {o, v});
  const TV R2 = cm(R + o * v, {o, o, v, v});
  auto E = [&](const char *spec, double alpha, const TV &A, const TV &Bt, double beta,
               const TV &C, bool cA = false, bool cB = false) {
    einsum(ctx, spec, alpha, A, Bt, beta, C, be, cA, cB);
  };
  make_tau(o, v, t1.p, t2.p, 1.0, w.tau.p(), s);                                     // :107
  const TV tau = w.tau.v;
  // t2 and tau are packed for the tensor cores several times, in different
  // orders: their maxima once each
  MaxHints hints(ctx, be);
  hints.add(t2.p, o * o * v * v);
  hints.add(tau.p, o * o * v * v);
  if (ctx.tape) {
    TapeOp op;
    op.kind = TapeOp::TAU;
    op.A = t1;
    op.B = t2;
    op.C = tau;
    op.o = o;
    op.v = v;
    ctx.tape->ops.push_back(op);
  }
  E("kcld,ilcd->ki", 1.0, B.L_ovov.v, tau, 0.0, w.Foo.v, true);                      // :111
  E("kcld,klad->ac", -1.0, B.L_ovov.v, tau, 0.0, w.Fvv.v, true);                     // :113
  E("kcld,ld->kc", 1.0, B.L_ovov.v, t1, 0.0, w.Fov.v, true);                         // :115

  E("ac,ic->ia", 1.0, w.Fvv.v, t1, 0.0, R1);                                         // :119
  E("ki,ka->ia", -1.0, w.Foo.v, t1, 1.0, R1);                                        // :121
  E("kc,kica->ia", 2.0, w.Fov.v, t2, 1.0, R1);                                       // :123
  E("kc,ikca->ia", -1.0, w.Fov.v, t2, 1.0, R1);                                      // :124
  E("kc,ic->ki", 1.0, w.Fov.v, t1, 0.0, w.Fovt1.v);                                  // :127
  E("ki,ka->ia", 1.0, w.Fovt1.v, t1, 1.0, R1);                                       // :128
  E("kcai,kc->ia", 2.0, B.ovvo, t1, 1.0, R1, true);                                  // :131
  E("kiac,kc->ia", -1.0, B.oovv, t1, 1.0, R1, true);                                 // :132
  // The reassociated list (not recorded for the adjoint, whose gradients flow
  // back through views of the eri) contracts each pair of terms over the same
  // index pattern once, with the combined integrals L_ovvv, L_ovoo.
  const bool combined = !literal && !ctx.tape;
  if (combined) {
    E("kdac,ikcd->ia", 1.0, B.l_ovvv(ctx), tau, 1.0, R1, true);                      // :134-135
    E("lcki,klac->ia", -1.0, B.l_ovoo(ctx), tau, 1.0, R1, true);                     // :137-138
  } else {
    E("kdac,ikcd->ia", 2.0, B.ovvv, tau, 1.0, R1, true);                             // :134
    E("kcad,ikcd->ia", -1.0, B.ovvv, tau, 1.0, R1, true);                            // :135
    E("lcki,klac->ia", -2.0, B.ovoo, tau, 1.0, R1, true);                            // :137
    E("kcli,klac->ia", 1.0, B.ovoo, tau, 1.0, R1, true);                             // :138
  }

  // T2.  X collects every term the reference wraps in PlusTranspose.
  if (literal) {
    E("kibc,ka->abic", -1.0, B.oovv, t1, 0.0, w.tmp_abic.v, true);                   // :144
    permute(ctx, "iacb->abic", 1.0, B.ovvv, 1.0, w.tmp_abic.v);                      // :145
    E("abic,jc->ijab", 1.0, w.tmp_abic.v, t1, 0.0, w.X.v);                           // :147
  } else {
    // :144-147 reassociated: sum_c [-sum_k (ki|bc) t1(k,a) + (ia|cb)] t1(j,c)
    //   = -sum_k t1(k,a) [sum_c (ki|bc) t1(j,c)] + sum_c (ia|cb) t1(j,c):
    // no v^3 o intermediate, no permuted copy of ovvv, 9x fewer FLOPs
    E("kibc,jc->kibj", 1.0, B.oovv, t1, 0.0, w.tmp_kibj.v, true);
    E("iacb,jc->ijab", 1.0, B.ovvv, t1, 0.0, w.X.v, true);
    E("kibj,ka->ijab", -1.0, w.tmp_kibj.v, t1, 1.0, w.X.v);
  }
  E("kcai,jc->akij", 1.0, B.ovvo, t1, 0.0, w.tmp_akij.v, true);                      // :152
  permute(ctx, "iajk->akij", 1.0, B.ovoo, 1.0, w.tmp_akij.v);                        // :153
  E("akij,kb->ijab", -1.0, w.tmp_akij.v, t1, 1.0, w.X.v);                            // :155
  permute(ctx, "ijab->ijab", 1.0, B.oovv_phys, 0.0, R2);                             // :158
  if (t2driver) axpby(o * o * v * v, 1.0, t2driver, 1.0, R2.p, s);                   // :159-160

  permute(ctx, "ki->ki", 1.0, w.Foo.v, 0.0, w.Loo.v);                                // :163
  if (combined) {
    E("lcki,lc->ki", 1.0, B.l_ovoo(ctx), t1, 1.0, w.Loo.v, true);                    // :164-165
  } else {
    E("lcki,lc->ki", 2.0, B.ovoo, t1, 1.0, w.Loo.v, true);                           // :164
    E("kcli,lc->ki", -1.0, B.ovoo, t1, 1.0, w.Loo.v, true);                          // :165
  }
  permute(ctx, "ac->ac", 1.0, w.Fvv.v, 0.0, w.Lvv.v);                                // :167
  if (combined) {
    E("kdac,kd->ac", 1.0, B.l_ovvv(ctx), t1, 1.0, w.Lvv.v, true);                    // :168-169
  } else {
    E("kdac,kd->ac", 2.0, B.ovvv, t1, 1.0, w.Lvv.v, true);                           // :168
    E("kcad,kd->ac", -1.0, B.ovvv, t1, 1.0, w.Lvv.v, true);                          // :169
  }

  permute(ctx, "klij->klij", 1.0, B.oooo, 0.0, w.Woooo.v);                           // :172
  E("lcki,jc->klij", 1.0, B.ovoo, t1, 1.0, w.Woooo.v, true);                         // :173
  E("kclj,ic->klij", 1.0, B.ovoo, t1, 1.0, w.Woooo.v, true);                         // :174
  E("kcld,ijcd->klij", 1.0, B.ovov, tau, 1.0, w.Woooo.v, true);                      // :175

  permute(ctx, "kcai->akic", 1.0, B.ovvo, 0.0, w.Wvoov.v);                           // :183
  E("kcad,id->akic", 1.0, B.ovvv, t1, 1.0, w.Wvoov.v, true);                         // :185
  E("kcli,la->akic", -1.0, B.ovoo, t1, 1.0, w.Wvoov.v, true);                        // :186
  E("ldkc,ilda->akic", -0.5, B.ovov, t2, 1.0, w.Wvoov.v, true);                      // :188
  E("lckd,ilad->akic", -0.5, B.ovov, t2, 1.0, w.Wvoov.v, true);                      // :190
  E("ldkc,ilad->akic", 1.0, B.ovov, t2, 1.0, w.Wvoov.v, true);                       // :192
  E("ldkc,id->lkci", 1.0, B.ovov, t1, 0.0, w.tmp_lkci.v, true);                      // :195
  E("lkci,la->akic", -1.0, w.tmp_lkci.v, t1, 1.0, w.Wvoov.v);                        // :196

  permute(ctx, "kiac->akci", 1.0, B.oovv, 0.0, w.Wvovo.v);                           // :200
  E("kdac,id->akci", 1.0, B.ovvv, t1, 1.0, w.Wvovo.v, true);                         // :202
  E("lcki,la->akci", -1.0, B.ovoo, t1, 1.0, w.Wvovo.v, true);                        // :203
  E("lckd,ilda->akci", -0.5, B.ovov, t2, 1.0, w.Wvovo.v, true);                      // :205
  E("lckd,id->lcki", 1.0, B.ovov, t1, 0.0, w.tmp_lcki.v, true);                      // :209
  E("lcki,la->akci", -1.0, w.tmp_lcki.v, t1, 1.0, w.Wvovo.v);                        // :210

  E("klij,klab->ijab", 1.0, w.Woooo.v, tau, 1.0, R2);                                // :214
  if (literal) {
    permute(ctx, "abcd->abcd", 1.0, B.vvvv, 0.0, w.Wvvvv.v);                         // :178
    E("kdac,kb->abcd", -1.0, B.ovvv, t1, 1.0, w.Wvvvv.v, true);                      // :179
    E("kcbd,ka->abcd", -1.0, B.ovvv, t1, 1.0, w.Wvvvv.v, true);                      // :180
    E("abcd,ijcd->ijab", 1.0, w.Wvvvv.v, tau, 1.0, R2);                              // :216
  } else {
    // sum_cd Wvvvv tau = vvvv tau - PlusTranspose(sum_k t1(k,a) Y(k,b,i,j)),
    // Y(k,b,i,j) = sum_cd (kc|bd) tau(i,j,c,d), using tau(i,j,c,d) = tau(j,i,d,c).
    // vvvv tau in its symmetric / antisymmetric form (a quarter of the FLOPs);
    // the adjoint's recorded forward keeps the plain contraction.
    if (ctx.tape) E("abcd,ijcd->ijab", 1.0, B.vvvv, tau, 1.0, R2, true);             // :216
    else ladder_pm(ctx, B, tau, R2.p, be);
    E("kcbd,ijcd->kbij", 1.0, B.ovvv, tau, 0.0, w.Yd.v, true);                       // :179-180
    E("ka,kbij->ijab", -1.0, t1, w.Yd.v, 1.0, w.X.v);
  }
  E("ac,ijcb->ijab", 1.0, w.Lvv.v, t2, 1.0, w.X.v);                                  // :218
  E("ki,kjab->ijab", -1.0, w.Loo.v, t2, 1.0, w.X.v);                                 // :220
  // Wvoov and Wvovo are complete: each feeds two of the ring contractions below
  hints.add(w.Wvoov.p(), o * o * v * v);
  hints.add(w.Wvovo.p(), o * o * v * v);
  E("akic,kjcb->ijab", 2.0, w.Wvoov.v, t2, 1.0, w.X.v);                              // :223
  E("akci,kjcb->ijab", -1.0, w.Wvovo.v, t2, 1.0, w.X.v);                             // :225
  E("akic,kjbc->ijab", -1.0, w.Wvoov.v, t2, 1.0, w.X.v);                             // :228
  E("bkci,kjac->ijab", -1.0, w.Wvovo.v, t2, 1.0, w.X.v);                             // :231
  plus_transpose(o, v, 1.0, w.X.p(), R2.p, s);                                       // :147-232
  if (ctx.tape) {
    TapeOp op;
    op.kind = TapeOp::PLUS_T;
    op.A = w.X.v;
    op.C = R2;
    op.o = o;
    op.v = v;
    ctx.tape->ops.push_back(op);
  }
}

// ---------------------------------------------------------------------------------------------

void rccsd_residual_delta(Ctx &ctx, const RccsdBlocks &B, const double *amp0, const double *amp1,
                          const double *damp, const RccsdWork &w0, Backend be, RccsdWork &w,
                          double *tau1, double *dR) {
  const int64_t o = B.o, v = B.v, n2 = o * o * v * v;
  cudaStream_t s = ctx.stream;
  double *a0 = const_cast<double *>(amp0), *a1 = const_cast<double *>(amp1);
  double *da = const_cast<double *>(damp);
  // base (T0), full (T1 = T0 + d) and change (d) of the amplitudes
  const TV t1_0 = cm(a0, {o, v});
  const TV t1_1 = cm(a1, {o, v}), t2_1 = cm(a1 + o * v, {o, o, v, v});
  const TV dt1 = cm(da, {o, v}), dt2 = cm(da + o * v, {o, o, v, v});
  const TV R1 = cm(dR, {o, v});
  const TV R2 = cm(dR + o * v, {o, o, v, v});
  auto E = [&](const char *spec, double alpha, const TV &A, const TV &Bt, double beta,
               const TV &C, bool cA = false, bool cB = false) {
    einsum(ctx, spec, alpha, A, Bt, beta, C, be, cA, cB);
  };
  // d(A B) = dA B1 + A0 dB for a product of two changing factors
  auto E2 = [&](const char *spec, double alpha, const TV &dA, const TV &B1, const TV &A0,
                const TV &dB, double beta, const TV &C) {
    E(spec, alpha, dA, B1, beta, C);
    E(spec, alpha, A0, dB, 1.0, C);
  };
  make_tau_delta(o, v, t1_0.p, dt1.p, dt2.p, w.tau.p(), s);
  const TV dtau = w.tau.v;
  SCESS_CUDA(cudaMemcpyAsync(tau1, w0.tau.p(), n2 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  axpby(n2, 1.0, dtau.p, 1.0, tau1, s);
  const TV tau_1 = cm(tau1, {o, o, v, v});
  // the changes and the new amplitudes, each packed several times
  MaxHints hints(ctx, be);
  hints.add(dt2.p, n2);
  hints.add(dtau.p, n2);
  hints.add(t2_1.p, n2);
  hints.add(tau_1.p, n2);

  E("kcld,ilcd->ki", 1.0, B.L_ovov.v, dtau, 0.0, w.Foo.v, true);                     // :111
  E("kcld,klad->ac", -1.0, B.L_ovov.v, dtau, 0.0, w.Fvv.v, true);                    // :113
  E("kcld,ld->kc", 1.0, B.L_ovov.v, dt1, 0.0, w.Fov.v, true);                        // :115

  E2("ac,ic->ia", 1.0, w.Fvv.v, t1_1, w0.Fvv.v, dt1, 0.0, R1);                       // :119
  E2("ki,ka->ia", -1.0, w.Foo.v, t1_1, w0.Foo.v, dt1, 1.0, R1);                      // :121
  E2("kc,kica->ia", 2.0, w.Fov.v, t2_1, w0.Fov.v, dt2, 1.0, R1);                     // :123
  E2("kc,ikca->ia", -1.0, w.Fov.v, t2_1, w0.Fov.v, dt2, 1.0, R1);                    // :124
  E2("kc,ic->ki", 1.0, w.Fov.v, t1_1, w0.Fov.v, dt1, 0.0, w.Fovt1.v);                // :127
  E2("ki,ka->ia", 1.0, w.Fovt1.v, t1_1, w0.Fovt1.v, dt1, 1.0, R1);                   // :128
  E("kcai,kc->ia", 2.0, B.ovvo, dt1, 1.0, R1, true);                                 // :131
  E("kiac,kc->ia", -1.0, B.oovv, dt1, 1.0, R1, true);                                // :132
  E("kdac,ikcd->ia", 1.0, B.l_ovvv(ctx), dtau, 1.0, R1, true);                       // :134-135
  E("lcki,klac->ia", -1.0, B.l_ovoo(ctx), dtau, 1.0, R1, true);                      // :137-138

  // T2 (reassociated list; the constant <ij|ab> and driver terms drop out)
  E("kibc,jc->kibj", 1.0, B.oovv, dt1, 0.0, w.tmp_kibj.v, true);                     // :144-147
  E("iacb,jc->ijab", 1.0, B.ovvv, dt1, 0.0, w.X.v, true);
  E2("kibj,ka->ijab", -1.0, w.tmp_kibj.v, t1_1, w0.tmp_kibj.v, dt1, 1.0, w.X.v);
  E("kcai,jc->akij", 1.0, B.ovvo, dt1, 0.0, w.tmp_akij.v, true);                     // :152-153
  E2("akij,kb->ijab", -1.0, w.tmp_akij.v, t1_1, w0.tmp_akij.v, dt1, 1.0, w.X.v);     // :155
  SCESS_CUDA(cudaMemsetAsync(R2.p, 0, n2 * sizeof(double), s));                      // :158-160

  permute(ctx, "ki->ki", 1.0, w.Foo.v, 0.0, w.Loo.v);                                // :163
  E("lcki,lc->ki", 1.0, B.l_ovoo(ctx), dt1, 1.0, w.Loo.v, true);                     // :164-165
  permute(ctx, "ac->ac", 1.0, w.Fvv.v, 0.0, w.Lvv.v);                                // :167
  E("kdac,kd->ac", 1.0, B.l_ovvv(ctx), dt1, 1.0, w.Lvv.v, true);                     // :168-169

  E("lcki,jc->klij", 1.0, B.ovoo, dt1, 0.0, w.Woooo.v, true);                        // :172-173
  E("kclj,ic->klij", 1.0, B.ovoo, dt1, 1.0, w.Woooo.v, true);                        // :174
  E("kcld,ijcd->klij", 1.0, B.ovov, dtau, 1.0, w.Woooo.v, true);                     // :175

  E("kcad,id->akic", 1.0, B.ovvv, dt1, 0.0, w.Wvoov.v, true);                        // :183-185
  E("kcli,la->akic", -1.0, B.ovoo, dt1, 1.0, w.Wvoov.v, true);                       // :186
  E("ldkc,ilda->akic", -0.5, B.ovov, dt2, 1.0, w.Wvoov.v, true);                     // :188
  E("lckd,ilad->akic", -0.5, B.ovov, dt2, 1.0, w.Wvoov.v, true);                     // :190
  E("ldkc,ilad->akic", 1.0, B.ovov, dt2, 1.0, w.Wvoov.v, true);                      // :192
  E("ldkc,id->lkci", 1.0, B.ovov, dt1, 0.0, w.tmp_lkci.v, true);                     // :195
  E2("lkci,la->akic", -1.0, w.tmp_lkci.v, t1_1, w0.tmp_lkci.v, dt1, 1.0, w.Wvoov.v); // :196

  E("kdac,id->akci", 1.0, B.ovvv, dt1, 0.0, w.Wvovo.v, true);                        // :200-202
  E("lcki,la->akci", -1.0, B.ovoo, dt1, 1.0, w.Wvovo.v, true);                       // :203
  E("lckd,ilda->akci", -0.5, B.ovov, dt2, 1.0, w.Wvovo.v, true);                     // :205
  E("lckd,id->lcki", 1.0, B.ovov, dt1, 0.0, w.tmp_lcki.v, true);                     // :209
  E2("lcki,la->akci", -1.0, w.tmp_lcki.v, t1_1, w0.tmp_lcki.v, dt1, 1.0, w.Wvovo.v); // :210

  E2("klij,klab->ijab", 1.0, w.Woooo.v, tau_1, w0.Woooo.v, dtau, 1.0, R2);           // :214
  // particle ladder with the T1 dressing folded in (as the reassociated list)
  ladder_pm(ctx, B, dtau, R2.p, be);                                                 // :216
  E("kcbd,ijcd->kbij", 1.0, B.ovvv, dtau, 0.0, w.Yd.v, true);                        // :179-180
  // d(t1 Yd) = dt1 Yd0 + t1_1 dYd
  E("ka,kbij->ijab", -1.0, dt1, w0.Yd.v, 1.0, w.X.v);
  E("ka,kbij->ijab", -1.0, t1_1, w.Yd.v, 1.0, w.X.v);
  E2("ac,ijcb->ijab", 1.0, w.Lvv.v, t2_1, w0.Lvv.v, dt2, 1.0, w.X.v);                // :218
  E2("ki,kjab->ijab", -1.0, w.Loo.v, t2_1, w0.Loo.v, dt2, 1.0, w.X.v);               // :220
  E2("akic,kjcb->ijab", 2.0, w.Wvoov.v, t2_1, w0.Wvoov.v, dt2, 1.0, w.X.v);          // :223
  E2("akci,kjcb->ijab", -1.0, w.Wvovo.v, t2_1, w0.Wvovo.v, dt2, 1.0, w.X.v);         // :225
  E2("akic,kjbc->ijab", -1.0, w.Wvoov.v, t2_1, w0.Wvoov.v, dt2, 1.0, w.X.v);         // :228
  E2("bkci,kjac->ijab", -1.0, w.Wvovo.v, t2_1, w0.Wvovo.v, dt2, 1.0, w.X.v);         // :231
  plus_transpose(o, v, 1.0, w.X.p(), R2.p, s);                                       // :147-232
}

// ---------------------------------------------------------------------------------------------

std::vector<double> full_piv_lu_solve(std::vector<double> A, std::vector<double> b, int n) {
  std::vector<int> rowp(n), colp(n);
  for (int i = 0; i < n; i++) rowp[i] = colp[i] = i;
  int nonzero = n;
  auto at = [&](int i, int j) -> double & { return A[(size_t)i * n + j]; };
  for (int k = 0; k < n; k++) {
    double best = -1.0;
    int bi = k, bj = k;
    for (int i = k; i < n; i++)
      for (int j = k; j < n; j++) {
        const double x = std::fabs(at(i, j));
        if (x > best) { best = x; bi = i; bj = j; }
      }
    if (best == 0.0) { nonzero = k; break; }
    if (bi != k) {
      for (int j = 0; j < n; j++) std::swap(at(k, j), at(bi, j));
      std::swap(rowp[k], rowp[bi]);
    }
    if (bj != k) {
      for (int i = 0; i < n; i++) std::swap(at(i, k), at(i, bj));
      std::swap(colp[k], colp[bj]);
    }
    for (int i = k + 1; i < n; i++) {
      at(i, k) /= at(k, k);
      for (int j = k + 1; j < n; j++) at(i, j) -= at(i, k) * at(k, j);
    }
  }
  double maxpiv = 0.0;
  for (int i = 0; i < nonzero; i++) maxpiv = std::max(maxpiv, std::fabs(at(i, i)));
  const double thresh = DBL_EPSILON * n;
  int rank = 0;
  for (int i = 0; i < nonzero; i++)
    if (std::fabs(at(i, i)) > thresh * maxpiv) rank++;
  std::vector<double> c(n), y(n, 0.0), x(n, 0.0);
  for (int i = 0; i < n; i++) c[i] = b[rowp[i]];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < std::min(i, rank); j++) c[i] -= at(i, j) * c[j];
  for (int i = rank - 1; i >= 0; i--) {
    double sum = c[i];
    for (int j = i + 1; j < rank; j++) sum -= at(i, j) * y[j];
    y[i] = sum / at(i, i);
  }
  for (int i = 0; i < n; i++) x[colp[i]] = y[i];
  return x;
}

std::vector<double> diis_coefficients(const std::vector<std::vector<double>> &gram) {
  const int n = (int)gram.size();
  const int m = n + 1;
  std::vector<double> B((size_t)m * m, -1.0);
  B[(size_t)n * m + n] = 0.0;
  double maxv = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      B[(size_t)i * m + j] = gram[i][j];
      maxv = std::max(maxv, std::fabs(gram[i][j]));
    }
  if (maxv > 0.0)
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) B[(size_t)i * m + j] /= maxv;
  std::vector<double> rhs(m, 0.0);
  rhs[n] = -1.0;
  std::vector<double> c = full_piv_lu_solve(B, rhs, m);
  c.resize(n);
  return c;
}

// ---------------------------------------------------------------------------------------------

RccsdState::RccsdState(Ctx &ctx, DTensor &&eri, int64_t nmo, int64_t nocc, const SolveInput &in,
                       const scess_rccsd_options &opts)
    : ctx_(ctx), eri_(std::move(eri)), opts_(opts) {
  B_.build(ctx, eri_.p(), nmo, nocc);
  init(in, opts);
}

RccsdState::RccsdState(Ctx &ctx, DTensor &&B, int64_t naux, int64_t nmo, int64_t nocc,
                       const SolveInput &in, const scess_rccsd_options &opts)
    : ctx_(ctx), dfB_(std::move(B)), naux_(naux), opts_(opts) {
  // mixed solves contract the regions on the tensor cores (~3e-7 relative per
  // integral), FP64 solves exactly
  B_.build_df(ctx, dfB_.p(), naux, nmo, nocc,
              opts.precision == SCESS_PRECISION_MIXED ? Backend::TENSOR : Backend::FP64);
  init(in, opts);
}

void RccsdState::init(const SolveInput &in, const scess_rccsd_options &opts) {
  Ctx &ctx = ctx_;
  const int64_t o = B_.o, v = B_.v, N = B_.N;
  n1_ = o * v;
  n2_ = o * o * v * v;
  n_ = n1_ + n2_;
  mixed_ = opts.precision == SCESS_PRECISION_MIXED;
  have_f12_ = in.f12_residual != nullptr;
  eps_ = DTensor({N});
  upload(ctx, eps_.p(), in.eps_host, N);
  amp_ = DTensor({n_});
  prev_ = DTensor({n_});
  R_ = DTensor({n_});
  if (in.f12_residual) {
    drv_ = DTensor({o, o, v, v});
    upload(ctx, drv_.p(), in.f12_residual, n2_);
  }
  if (in.f12_energy) {
    DTensor e12({o, o, v, v});
    upload(ctx, e12.p(), in.f12_energy, n2_);
    Lf12_ = DTensor({o, o, v, v});
    permute(ctx, "ijab->ijab", 2.0, e12.v, 0.0, Lf12_.v);                            // :95-96
    permute(ctx, "ijba->ijab", -1.0, e12.v, 1.0, Lf12_.v);
    ctx.sync();
  }
  maxv_ = std::max(1, opts.max_diis_vectors);
  diis_amp_.alloc((size_t)maxv_ * n_ * sizeof(double));
  diis_err_.alloc((size_t)maxv_ * n_ * sizeof(double));
  vecptr_.alloc((size_t)maxv_ * sizeof(double *));
  coefd_.alloc((size_t)(maxv_ + 1) * sizeof(double));
  w_.alloc(o, v, !mixed_);
  have_wvvvv_ = !mixed_;
  phase_ = mixed_ ? Phase::MIXED : Phase::FP64;
  std::memset(&res_, 0, sizeof(res_));
  SCESS_CUDA(cudaEventCreate(&ev0_));
  SCESS_CUDA(cudaEventCreate(&ev1_));
}

RccsdState::~RccsdState() {
  cudaEventDestroy(ev0_);
  cudaEventDestroy(ev1_);
}

void RccsdState::mp2_guess() {
  // t1 = 0, t2 = (<ij|ab> + f12 residual) / eijab                                    :334-339
  const int64_t o = B_.o, v = B_.v;
  cudaStream_t s = ctx_.stream;
  SCESS_CUDA(cudaMemsetAsync(R_.p(), 0, n1_ * sizeof(double), s));
  permute(ctx_, "ijab->ijab", 1.0, B_.oovv_phys, 0.0, cm(R_.p() + n1_, {o, o, v, v}));
  if (drv_.p()) axpby(n2_, 1.0, drv_.p(), 1.0, R_.p() + n1_, s);
  divide_denominators(o, v, eps_.p(), R_.p(), R_.p() + n1_, amp_.p(), amp_.p() + n1_, s);
  reset_history();
}

void RccsdState::set_amplitudes(const double *t1, const double *t2) {
  upload(ctx_, amp_.p(), t1, n1_);
  upload(ctx_, amp_.p() + n1_, t2, n2_);
  reset_history();
}

void RccsdState::get_amplitudes(double *t1, double *t2) {
  if (t1) download(ctx_, t1, amp_.p(), n1_);
  if (t2) download(ctx_, t2, amp_.p() + n1_, n2_);
}

void RccsdState::reset_history() {
  order_.clear();
  gram_.clear();
  E_last_ = DBL_MAX;
  it_ = 0;
  phase_start_ = 0;
  fp64_iters_ = 0;
  phase_ = mixed_ ? Phase::MIXED : Phase::FP64;
  converged_ = false;
  std::memset(&res_, 0, sizeof(res_));
}

double RccsdState::energy_of_amplitudes() {
  const int64_t o = B_.o, v = B_.v;
  cudaStream_t s = ctx_.stream;
  tau_energy(o, v, B_.L_oovv.p(), amp_.p(), amp_.p() + n1_, ctx_.partials, ctx_.dscalars, s);
  if (Lf12_.p()) dot(n2_, Lf12_.p(), amp_.p() + n1_, ctx_.partials, ctx_.dscalars + 1, s);
  SCESS_CUDA(cudaMemcpyAsync(ctx_.hscalars, ctx_.dscalars, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  ctx_.sync();
  return ctx_.hscalars[0] + (Lf12_.p() ? ctx_.hscalars[1] : 0.0);
}

bool RccsdState::iterate(int max_steps, const Control &ctl) {
  const int64_t o = B_.o, v = B_.v;
  cudaStream_t s = ctx_.stream;
  double *t1 = amp_.p(), *t2 = amp_.p() + n1_;
  SCESS_CUDA(cudaEventRecord(ev0_, s));
  int steps = 0;
  while (steps < max_steps && it_ < opts_.max_iterations && !converged_) {
    ctl.poll();                                                                       // :346
    SCESS_CUDA(cudaMemcpyAsync(prev_.p(), amp_.p(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    const Phase ph = phase_;
    if (ph == Phase::MIXED) {
      rccsd_residual(ctx_, B_, amp_.p(), drv_.p(), Backend::MIXED, w_, R_.p());       // :350
    } else if (ph == Phase::FP64) {
      if (!have_wvvvv_) {
        w_.Wvvvv = DTensor({v, v, v, v});
        have_wvvvv_ = true;
      }
      rccsd_residual(ctx_, B_, amp_.p(), drv_.p(), Backend::FP64, w_, R_.p());
    } else if (ph == Phase::REFINED) {
      // R = R0 + dR(T0, T - T0)
      SCESS_CUDA(cudaMemcpyAsync(damp_.p(), amp_.p(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
      axpby(n_, -1.0, amp0_.p(), 1.0, damp_.p(), s);
      rccsd_residual_delta(ctx_, B_, amp0_.p(), amp_.p(), damp_.p(), w0_, Backend::MIXED, w_,
                           tau1_.p(), R_.p());
      axpby(n_, 1.0, R0_.p(), 1.0, R_.p(), s);
    } else {  // BASE, CONFIRM: FP64, the reassociated list, intermediates kept in w0_
      if (!amp0_.p()) {
        w0_.alloc(o, v, false);
        amp0_ = DTensor({n_});
        R0_ = DTensor({n_});
        damp_ = DTensor({n_});
        tau1_ = DTensor({o, o, v, v});
      }
      rccsd_residual(ctx_, B_, amp_.p(), drv_.p(), Backend::FP64, w0_, R_.p(),
                     ResidualList::REASSOCIATED);
      SCESS_CUDA(cudaMemcpyAsync(amp0_.p(), amp_.p(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
      SCESS_CUDA(cudaMemcpyAsync(R0_.p(), R_.p(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    divide_denominators(o, v, eps_.p(), R_.p(), R_.p() + n1_, t1, t2, s);

    // AmplitudeDIIS::Extrapolate(updated, change)                                    :246-274
    int slot;
    if ((int)order_.size() < maxv_) {
      slot = (int)order_.size();
    } else {
      slot = order_.front();
      order_.pop_front();
      gram_.erase(gram_.begin());
      for (auto &row : gram_) row.erase(row.begin());
    }
    double *va = diis_amp_.d() + (size_t)slot * n_;
    double *ve = diis_err_.d() + (size_t)slot * n_;
    SCESS_CUDA(cudaMemcpyAsync(va, amp_.p(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    SCESS_CUDA(cudaMemcpyAsync(ve, amp_.p(), n_ * sizeof(double), cudaMemcpyDeviceToDevice, s));
    axpby(n_, -1.0, prev_.p(), 1.0, ve, s);                                           // :352
    order_.push_back(slot);
    const int nv = (int)order_.size();
    for (int q = 0; q < nv; q++)
      dot(n_, diis_err_.d() + (size_t)order_[q] * n_, ve, ctx_.partials, ctx_.dscalars + q, s);
    SCESS_CUDA(cudaMemcpyAsync(ctx_.hscalars, ctx_.dscalars, nv * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    ctx_.sync();
    for (int q = 0; q < nv - 1; q++) gram_[q].push_back(ctx_.hscalars[q]);
    gram_.emplace_back(ctx_.hscalars, ctx_.hscalars + nv);
    const double errdot = ctx_.hscalars[nv - 1];
    if (it_ - phase_start_ >= opts_.diis_start) {                                    // :354-357
      if (it_ - phase_start_ == opts_.diis_start) ctx_.logf(1, "Turning on DIIS");
      std::vector<double> c = diis_coefficients(gram_);
      std::vector<const double *> hptr(nv);
      for (int q = 0; q < nv; q++) hptr[q] = diis_amp_.d() + (size_t)order_[q] * n_;
      SCESS_CUDA(cudaMemcpyAsync(vecptr_.as<void>(), hptr.data(), nv * sizeof(double *),
                                 cudaMemcpyHostToDevice, s));
      SCESS_CUDA(cudaMemcpyAsync(coefd_.d(), c.data(), nv * sizeof(double), cudaMemcpyHostToDevice, s));
      linear_combination(n_, nv, vecptr_.as<const double *>(), coefd_.d(), amp_.p(), s);
      ctx_.sync();  // hptr / c are host buffers of this scope
    }
    const double E = energy_of_amplitudes();                                          // :361
    const double dE = std::fabs(E - E_last_);                                         // :362
    const double rms = std::sqrt(errdot) / std::sqrt((double)n_);                     // :363
    E_last_ = E;
    if (!std::isfinite(E)) throw Error(SCESS_ERR_INVALID, "non-finite CCSD energy (diverging amplitudes)");
    static const char *const kTag[] = {"", "   [mixed]", "   [fp64 base]", "   [refined]",
                                       "   [fp64]"};
    ctx_.logf(1, "   CCSD(%d): E(corr) = %.12g      dE = %.12g      rms(dt) = %.12g%s", it_, E,
              dE, rms, kTag[(int)ph]);
    if (opts_.history) {
      opts_.history[3 * it_ + 0] = E;
      opts_.history[3 * it_ + 1] = dE;
      opts_.history[3 * it_ + 2] = rms;
    }
    if (opts_.checkpoint_capacity > 0 && opts_.checkpoint_t1 && opts_.checkpoint_t2) {
      const int sl = it_ % opts_.checkpoint_capacity;
      download(ctx_, opts_.checkpoint_t1 + (size_t)sl * n1_, t1, n1_);
      download(ctx_, opts_.checkpoint_t2 + (size_t)sl * n2_, t2, n2_);
    }
    res_.last_dE = dE;
    res_.last_rms = rms;
    const bool fp64_it = ph == Phase::FP64 || ph == Phase::BASE || ph == Phase::CONFIRM;
    if (fp64_it) fp64_iters_++;
    else res_.mixed_iterations++;
    it_++;
    steps++;
    res_.iterations = it_;
    res_.fp64_iterations = fp64_iters_;
    const bool meets = dE < opts_.energy_convergence && rms < opts_.amplitude_convergence;  // :370
    switch (ph) {
      case Phase::FP64:
        converged_ = meets;
        break;
      case Phase::MIXED:
        if (dE < opts_.mixed_energy_switch && rms < opts_.mixed_amplitude_switch) {
          // refinement from the mixed amplitudes with a fresh DIIS subspace
          phase_ = Phase::BASE;
          phase_start_ = it_;
          order_.clear();
          gram_.clear();
          ctx_.logf(1, "Mixed-precision phase done; refinement from an FP64 base");
        }
        break;
      case Phase::BASE:
        phase_ = Phase::REFINED;
        break;
      case Phase::REFINED:
        if (meets) phase_ = Phase::CONFIRM;
        break;
      case Phase::CONFIRM:
        if (meets && fp64_iters_ >= std::max(1, opts_.refine_sweeps)) {
          converged_ = true;
        } else {
          // this FP64 evaluation is the new base (its residual and
          // intermediates at its input amplitudes are kept)
          phase_ = Phase::REFINED;
          ctx_.logf(1, "FP64 check not met; refining from it");
        }
        break;
    }
  }
  SCESS_CUDA(cudaEventRecord(ev1_, s));
  SCESS_CUDA(cudaEventSynchronize(ev1_));
  float ms = 0.0f;
  SCESS_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
  last_device_ms_ = ms;
  if (mixed_ && ctx_.tc) ctx_.tc->check_error();
  res_.converged = converged_ ? 1 : 0;
  res_.E_CCSD = converged_ ? E_last_ : 0.0;
  return converged_;
}

double RccsdState::coupling_energy() {
  if (!Lf12_.p()) return 0.0;
  dot(n2_, Lf12_.p(), amp_.p() + n1_, ctx_.partials, ctx_.dscalars, ctx_.stream);
  SCESS_CUDA(cudaMemcpyAsync(ctx_.hscalars, ctx_.dscalars, sizeof(double), cudaMemcpyDeviceToHost, ctx_.stream));
  ctx_.sync();
  return ctx_.hscalars[0];
}

void rccsd_solve(Ctx &ctx, RccsdState &st, const Control &ctl, double *t1_out, double *t2_out,
                 scess_rccsd_result *res) {
  ctx.logf(0, st.has_f12()
                  ? "--- Closed-shell CCSD with F12 geminals (CCSD-F12b) with DIIS acceleration ---"
                  : "--- Closed-shell Coupled Cluster Singles & Doubles (CCSD) with DIIS acceleration ---");
  const bool conv = st.iterate(st.options().max_iterations, ctl);
  *res = st.result();
  if (!conv) {                                                                        // :376-380
    ctx.logf(0, "!!! CCSD procedure failed to converge !!!");
    res->E_CCSD = 0.0;
    return;
  }
  res->E_F12_Coupling = st.coupling_energy();                                         // :383
  st.get_amplitudes(t1_out, t2_out);
  ctx.logf(0, "---- CCSD procedure converged! ----");
  ctx.logf(0, "E(CCSD correlation) = %.12g hartrees", res->E_CCSD);
}

}  // namespace scess
