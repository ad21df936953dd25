/*
 * C + OpenMP restatement of SCESS's closed-shell (T), RCCSD_TriplesCorrection
 * (src/Quantum/CC/RCCSD_T.cpp:17-168).  TEST INFRASTRUCTURE: it is the timed
 * CPU baseline and a second oracle for the (T) energy; nothing in the product
 * links it.
 *
 * Same structure as the reference: the P/R/S/Q repack (:30-56), per unique
 * triple a >= b >= c (:109-114) the matrix products of GetW (:62-68) and the
 * rank-one GetV (:70-75), Symmetrise through a scratch array (:78-106), r3,
 * the degeneracy weight and the energy (:133-157), a dynamic parallel loop
 * over the triples with per-thread o^3 buffers (:116-122) and the factor 2
 * (:167).  The reference's matrix products go to BLAS dgemm; here they are
 * plain loops ordered for unit-stride inner loops (the compiler vectorises
 * them).  Arrays are column-major like the reference's Eigen tensors.
 *
 * triples over a in [a_begin, a_end) only, so that a caller can time a slice.
 */
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t idx;

static void get_w(idx o, idx v, const double *P, const double *Q, const double *R,
                  const double *t2, idx a, idx b, idx c, double *out) {
  const idx o2 = o * o;
  const double *Pab = P + o * v * (a + v * b); /* o x v, (i, f) */
  const double *Qc = Q + v * o2 * c;           /* v x o^2, (f, jk) */
  const double *Ra = R + o2 * o * a;           /* o^2 x o, (ij, m) */
  const double *tbc = t2 + o2 * (b + v * c);   /* o x o, (m, k) */
  /* w(i, jk) = sum_f P(i,f,a,b) Q(f,j,k,c), four jk columns at a time      :64-65 */
  idx jk = 0;
  for (; jk + 4 <= o2; jk += 4) {
    double *w0 = out + o * jk, *w1 = w0 + o, *w2 = w1 + o, *w3 = w2 + o;
    for (idx i = 0; i < 4 * o; i++) w0[i] = 0.0;
    const double *q0 = Qc + v * jk, *q1 = q0 + v, *q2 = q1 + v, *q3 = q2 + v;
    for (idx f = 0; f < v; f++) {
      const double a0 = q0[f], a1 = q1[f], a2 = q2[f], a3 = q3[f];
      const double *p = Pab + o * f;
      for (idx i = 0; i < o; i++) {
        const double pi = p[i];
        w0[i] += pi * a0;
        w1[i] += pi * a1;
        w2[i] += pi * a2;
        w3[i] += pi * a3;
      }
    }
  }
  for (; jk < o2; jk++) {
    double *w = out + o * jk;
    for (idx i = 0; i < o; i++) w[i] = 0.0;
    const double *q = Qc + v * jk;
    for (idx f = 0; f < v; f++) {
      const double qf = q[f];
      const double *p = Pab + o * f;
      for (idx i = 0; i < o; i++) w[i] += p[i] * qf;
    }
  }
  /* w(ij, k) -= sum_m R(i,j,m,a) t2(m,k,b,c)                                :66-67 */
  for (idx k = 0; k < o; k++) {
    double *w = out + o2 * k;
    for (idx m = 0; m < o; m++) {
      const double t = tbc[m + o * k];
      const double *r = Ra + o2 * m;
      for (idx ij = 0; ij < o2; ij++) w[ij] -= r[ij] * t;
    }
  }
}

static void get_v(idx o, idx v, const double *S, const double *t1, idx a, idx b, idx c,
                  double *out) {
  const idx o2 = o * o;
  const double *Sab = S + o2 * (a + v * b);
  /* v(ij, k) = t1(k,c) / 2 * S(i,j,a,b)                                     :70-75 */
  for (idx k = 0; k < o; k++) {
    const double s = 0.5 * t1[k + o * c];
    for (idx ij = 0; ij < o2; ij++) out[ij + o2 * k] = s * Sab[ij];
  }
}

#define IDX(i, j, k) ((i) + o * (j) + o2 * (k))

/* Symmetrise (:78-106): X_ijk^abc + X_ikj^acb + X_jik^bac + X_jki^bca + X_kij^cab + X_kji^cba */
static void symmetrise_w(idx o, idx v, const double *P, const double *Q, const double *R,
                         const double *t2, idx a, idx b, idx c, double *out, double *sc) {
  const idx o2 = o * o;
  get_w(o, v, P, Q, R, t2, a, b, c, out);
  get_w(o, v, P, Q, R, t2, a, c, b, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(i, k, j)];
  get_w(o, v, P, Q, R, t2, b, a, c, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(j, i, k)];
  get_w(o, v, P, Q, R, t2, b, c, a, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(j, k, i)];
  get_w(o, v, P, Q, R, t2, c, a, b, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(k, i, j)];
  get_w(o, v, P, Q, R, t2, c, b, a, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(k, j, i)];
}

static void symmetrise_v(idx o, idx v, const double *S, const double *t1, idx a, idx b, idx c,
                         double *out, double *sc) {
  const idx o2 = o * o;
  get_v(o, v, S, t1, a, b, c, out);
  get_v(o, v, S, t1, a, c, b, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(i, k, j)];
  get_v(o, v, S, t1, b, a, c, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(j, i, k)];
  get_v(o, v, S, t1, b, c, a, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(j, k, i)];
  get_v(o, v, S, t1, c, a, b, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(k, i, j)];
  get_v(o, v, S, t1, c, b, a, sc);
  for (idx k = 0; k < o; k++)
    for (idx j = 0; j < o; j++)
      for (idx i = 0; i < o; i++) out[IDX(i, j, k)] += sc[IDX(k, j, i)];
}

/* Returns E_(T) restricted to leading virtuals a in [a_begin, a_end) (already x2). */
double scess_ref_triples(const double *eri, const double *eps, idx nmo, idx o, const double *t1,
                         const double *t2, idx a_begin, idx a_end, int nthreads) {
  const idx v = nmo - o, N = nmo, N2 = N * N, N3 = N2 * N, o2 = o * o, o3 = o2 * o;
  double *P = (double *)malloc(sizeof(double) * o * v * v * v);
  double *R = (double *)malloc(sizeof(double) * o3 * v);
  double *S = (double *)malloc(sizeof(double) * o2 * v * v);
  double *Q = (double *)malloc(sizeof(double) * v * o2 * v);
  if (!P || !R || !S || !Q) {
    free(P); free(R); free(S); free(Q);
    return 0.0;
  }
  if (nthreads > 0) omp_set_num_threads(nthreads);
  /* repack, :37-56 */
#pragma omp parallel for schedule(static)
  for (idx b = 0; b < v; b++)
    for (idx a = 0; a < v; a++)
      for (idx f = 0; f < v; f++)
        for (idx i = 0; i < o; i++)
          P[i + o * (f + v * (a + v * b))] = eri[i + N * (o + b) + N2 * (o + a) + N3 * (o + f)];
#pragma omp parallel for schedule(static)
  for (idx a = 0; a < v; a++)
    for (idx m = 0; m < o; m++)
      for (idx j = 0; j < o; j++)
        for (idx i = 0; i < o; i++)
          R[i + o * (j + o * (m + o * a))] = eri[i + N * m + N2 * (o + a) + N3 * j];
#pragma omp parallel for schedule(static)
  for (idx b = 0; b < v; b++)
    for (idx a = 0; a < v; a++)
      for (idx j = 0; j < o; j++)
        for (idx i = 0; i < o; i++)
          S[i + o * (j + o * (a + v * b))] = eri[i + N * j + N2 * (o + a) + N3 * (o + b)];
#pragma omp parallel for schedule(static)
  for (idx c = 0; c < v; c++)
    for (idx k = 0; k < o; k++)
      for (idx j = 0; j < o; j++)
        for (idx f = 0; f < v; f++)
          Q[f + v * (j + o * (k + o * c))] = t2[k + o * (j + o * (c + v * f))];

  /* the unique triples a >= b >= c with a in [a_begin, a_end), :109-114 */
  idx ntrip = 0;
  for (idx a = a_begin; a < a_end; a++) ntrip += (a + 1) * (a + 2) / 2;
  idx *trip = (idx *)malloc(sizeof(idx) * 3 * (ntrip > 0 ? ntrip : 1));
  idx n = 0;
  for (idx a = a_begin; a < a_end; a++)
    for (idx b = 0; b <= a; b++)
      for (idx c = 0; c <= b; c++) {
        trip[3 * n] = a;
        trip[3 * n + 1] = b;
        trip[3 * n + 2] = c;
        n++;
      }
  double energy = 0.0;
#pragma omp parallel reduction(+ : energy)
  {
    double *W = (double *)malloc(sizeof(double) * 4 * o3);  /* W, V, Z, scratch :116-119 */
    double *V = W + o3, *Z = V + o3, *sc = Z + o3;
#pragma omp for schedule(dynamic, 1)
    for (idx t = 0; t < ntrip; t++) {
      const idx a = trip[3 * t], b = trip[3 * t + 1], c = trip[3 * t + 2];
      symmetrise_w(o, v, P, Q, R, t2, a, b, c, W, sc);
      symmetrise_v(o, v, S, t1, a, b, c, V, sc);
      double deg = 1.0;                                            /* :135-139 */
      if (a == c) deg = 6.0;
      else if (a == b || b == c) deg = 2.0;
      for (idx q = 0; q < o3; q++) sc[q] = W[q] + V[q];            /* :145-146 */
      const double ev = eps[o + a] + eps[o + b] + eps[o + c];
      double e = 0.0;
      for (idx k = 0; k < o; k++)
        for (idx j = 0; j < o; j++)
          for (idx i = 0; i < o; i++) {
            const double r3 = 4.0 * sc[IDX(i, j, k)] + sc[IDX(k, i, j)] + sc[IDX(j, k, i)] -
                              2.0 * sc[IDX(k, j, i)] - 2.0 * sc[IDX(i, k, j)] -
                              2.0 * sc[IDX(j, i, k)];                 /* :152-154 */
            const double d3 = (eps[i] + eps[j] + eps[k] - ev) * deg; /* :155 */
            e += W[IDX(i, j, k)] * r3 / d3;                           /* :156 */
          }
      energy += e;
    }
    free(W);
  }
  free(trip);
  free(P);
  free(R);
  free(S);
  free(Q);
  return 2.0 * energy; /* :167 */
}
