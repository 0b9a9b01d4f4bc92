/*
 * CPU restatement of the reference RGF sweep -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain C99 + OpenMP (parallel over independent (E, k) points), complex128,
 * column-major n x n blocks.  It follows, step for step:
 *   sancho                    src/cuda_rgf_mod.f90:657-765 (src/rgf_mod.f90:482-568)
 *   cuda_rgf_constblocksize   src/cuda_rgf_mod.f90:53-413, with G^> = G^< + G - G^+
 *                             in every slab (what produced test_cnt/pdos0000.dat)
 * plus the Caroli transmission Tr[Gam_R G_N1 Gam_L G_N1^+].  Block products are
 * loops over split real / imaginary planes, four columns at a time, and inverses
 * Gauss-Jordan with partial pivoting: it
 * stands in for the reference's CPU build (no Fortran compiler exists on
 * either machine) as the timed CPU baseline and as a second checker.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

static const double BOLTZ = 8.61734e-05;

/* C = op(A) op(B)  (op: 'N' or 'C'), all n x n column-major (n <= 512).  The operands are
 * first split into real and imaginary planes (op applied), so the inner loop is plain real
 * multiply-adds that the compiler vectorises; four columns of C are formed together so
 * that each loaded entry of op(A) feeds four complex multiply-adds from L1.  Every C(i, j)
 * accumulates over k = 0 .. n-1 in order.  ta, tb hold 2 n^2 doubles each. */
static void gemm(int n, char opa, const cplx* A, char opb, const cplx* B, cplx* C, cplx* ta,
                 cplx* tb) {
  const size_t nn = (size_t)n * n;
  double* restrict ar = (double*)ta;
  double* restrict ai = ar + nn;
  double* restrict br = (double*)tb;
  double* restrict bi = br + nn;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const cplx x = opa == 'C' ? conj(A[j + (size_t)i * n]) : A[i + (size_t)j * n];
      const cplx y = opb == 'C' ? conj(B[j + (size_t)i * n]) : B[i + (size_t)j * n];
      ar[i + (size_t)j * n] = creal(x);
      ai[i + (size_t)j * n] = cimag(x);
      br[i + (size_t)j * n] = creal(y);
      bi[i + (size_t)j * n] = cimag(y);
    }
  enum { NJ = 4 };
  double cr[NJ][512], ci[NJ][512];
  for (int j0 = 0; j0 < n; j0 += NJ) {
    const int nj = n - j0 < NJ ? n - j0 : NJ;
    for (int q = 0; q < nj; ++q)
      for (int i = 0; i < n; ++i) cr[q][i] = ci[q][i] = 0.0;
    for (int k = 0; k < n; ++k) {
      const double* restrict xr = ar + (size_t)k * n;
      const double* restrict xi = ai + (size_t)k * n;
      for (int q = 0; q < nj; ++q) {
        const double yr = br[k + (size_t)(j0 + q) * n], yi = bi[k + (size_t)(j0 + q) * n];
        double* restrict zr = cr[q];
        double* restrict zi = ci[q];
        for (int i = 0; i < n; ++i) {
          zr[i] += xr[i] * yr - xi[i] * yi;
          zi[i] += xr[i] * yi + xi[i] * yr;
        }
      }
    }
    for (int q = 0; q < nj; ++q)
      for (int i = 0; i < n; ++i) C[i + (size_t)(j0 + q) * n] = cr[q][i] + I * ci[q][i];
  }
}

/* in-place inverse, Gauss-Jordan with row pivoting (|re|+|im| pivot measure) */
static int invert(int n, cplx* X, int* perm) {
  int bad = 0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1.0;
    for (int i = k; i < n; ++i) {
      const cplx v = X[i + (size_t)k * n];
      const double m = fabs(creal(v)) + fabs(cimag(v));
      if (m > best) { best = m; p = i; }
    }
    if (!(best > 0.0)) bad = 1;
    perm[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) {
        const cplx t = X[k + (size_t)j * n];
        X[k + (size_t)j * n] = X[p + (size_t)j * n];
        X[p + (size_t)j * n] = t;
      }
    const cplx inv = best > 0.0 ? 1.0 / X[k + (size_t)k * n] : 0.0;
    for (int j = 0; j < n; ++j) X[k + (size_t)j * n] *= inv;
    X[k + (size_t)k * n] = inv;
    for (int j = 0; j < n; ++j) {
      if (j == k) continue;
      const cplx r = X[k + (size_t)j * n];
      cplx* restrict col = X + (size_t)j * n;
      const cplx* restrict colk = X + (size_t)k * n;
      /* all rows, then row k put back: the same operations on rows i != k, in a loop
         without a branch */
      for (int i = 0; i < n; ++i) col[i] -= colk[i] * r;
      col[k] = r;
    }
    for (int i = 0; i < n; ++i)
      if (i != k) X[i + (size_t)k * n] *= -inv;
  }
  for (int k = n - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = 0; i < n; ++i) {
        const cplx t = X[i + (size_t)k * n];
        X[i + (size_t)k * n] = X[i + (size_t)p * n];
        X[i + (size_t)p * n] = t;
      }
  }
  return bad;
}

typedef struct {
  int n;
  cplx *A, *B, *C, *D, *ta, *tb, *HBB, *HSS, *H10, *H01;
  int* perm;
} Work;

static void work_init(Work* w, int n) {
  const size_t b = (size_t)n * n;
  w->n = n;
  w->A = malloc(sizeof(cplx) * b * 10);
  w->B = w->A + b; w->C = w->B + b; w->D = w->C + b; w->ta = w->D + b; w->tb = w->ta + b;
  w->HBB = w->tb + b; w->HSS = w->HBB + b; w->H10 = w->HSS + b; w->H01 = w->H10 + b;
  w->perm = malloc(sizeof(int) * n);
}
static void work_free(Work* w) { free(w->A); free(w->perm); }

static void dag(int n, const cplx* X, cplx* Y) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) Y[i + (size_t)j * n] = conj(X[j + (size_t)i * n]);
}

/* G00 (surface) of the decimation (src/cuda_rgf_mod.f90:657-765); returns iterations */
static int sancho(Work* w, double E, double eta, double tol, int nmax, const cplx* H00,
                  const cplx* H10, int dag_in, cplx* G00, int* bad) {
  const int n = w->n;
  const size_t b = (size_t)n * n;
  const cplx z = E + I * eta;
  memcpy(w->HBB, H00, sizeof(cplx) * b);
  memcpy(w->HSS, H00, sizeof(cplx) * b);
  if (dag_in) { dag(n, H10, w->H10); memcpy(w->H01, H10, sizeof(cplx) * b); }
  else { memcpy(w->H10, H10, sizeof(cplx) * b); dag(n, H10, w->H01); }
  int it;
  for (it = 1; it <= nmax; ++it) {
    for (size_t e = 0; e < b; ++e) w->A[e] = -w->HBB[e];
    for (int i = 0; i < n; ++i) w->A[i + (size_t)i * n] += z;
    *bad |= invert(n, w->A, w->perm);
    gemm(n, 'N', w->A, 'N', w->H10, w->B, w->ta, w->tb);
    gemm(n, 'N', w->H01, 'N', w->B, w->C, w->ta, w->tb);
    for (size_t e = 0; e < b; ++e) { w->HSS[e] += w->C[e]; w->HBB[e] += w->C[e]; }
    gemm(n, 'N', w->H10, 'N', w->B, w->C, w->ta, w->tb);
    gemm(n, 'N', w->A, 'N', w->H01, w->B, w->ta, w->tb);
    gemm(n, 'N', w->H10, 'N', w->B, w->A, w->ta, w->tb);
    memcpy(w->H10, w->C, sizeof(cplx) * b);
    for (size_t e = 0; e < b; ++e) w->HBB[e] += w->A[e];
    gemm(n, 'N', w->H01, 'N', w->B, w->C, w->ta, w->tb);
    memcpy(w->H01, w->C, sizeof(cplx) * b);
    double err = 0.0;
    for (size_t e = 0; e < b; ++e) err += cabs(w->C[e]);
    if (err < tol) break;
  }
  if (it > nmax) it = nmax;
  for (size_t e = 0; e < b; ++e) G00[e] = -w->HSS[e];
  for (int i = 0; i < n; ++i) G00[i + (size_t)i * n] += z;
  *bad |= invert(n, G00, w->perm);
  return it;
}

static double ferm(double a) { return 1.0 / (1.0 + exp(a)); }

/* Re Tr[X Y] */
static double trace_prod(int n, const cplx* X, const cplx* Y) {
  double s = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) s += creal(X[i + (size_t)j * n] * Y[j + (size_t)i * n]);
  return s;
}

/* one (E, k) point of the sweep; outputs for this point only */
static void point(Work* w, int nx, double E, const cplx* H0, const cplx* H10, double eta_lead,
                  double eta_int, double tol, int nmax, double fl, double fr, double fe,
                  cplx* gl, cplx* gln, cplx* s /* 12 blocks */, double* T, double* tr,
                  double* tre, cplx* dgr, cplx* dgl, int* status, int* iters) {
  const int n = w->n;
  const size_t b = (size_t)n * n;
  const cplx z = E + I * eta_int;
  cplx *SigL = s, *GamL = s + b, *SigR = s + 2 * b, *GamR = s + 3 * b, *Pc = s + 4 * b;
  cplx *G = s + 5 * b, *Gn = s + 6 * b, *X = s + 7 * b, *Y = s + 8 * b, *Z = s + 9 * b;
  cplx *V = s + 10 * b, *U = s + 11 * b;
  int bad = 0;
  /* left contact (src/cuda_rgf_mod.f90:90-134) */
  iters[0] = sancho(w, E, eta_lead, tol, nmax, H0, H10, 1, X, &bad);
  gemm(n, 'N', H10, 'N', X, Y, w->ta, w->tb);
  gemm(n, 'N', Y, 'C', H10, SigL, w->ta, w->tb);
  for (size_t e = 0; e < b; ++e) gl[e] = -H0[e] - SigL[e];
  for (int i = 0; i < n; ++i) gl[i + (size_t)i * n] += z;
  bad |= invert(n, gl, w->perm);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      GamL[i + (size_t)j * n] = -(SigL[i + (size_t)j * n] - conj(SigL[j + (size_t)i * n]));
  for (size_t e = 0; e < b; ++e) V[e] = GamL[e] * fl;
  gemm(n, 'N', gl, 'N', V, Y, w->ta, w->tb);
  gemm(n, 'N', Y, 'C', gl, gln, w->ta, w->tb);
  memcpy(Pc, gl, sizeof(cplx) * b);
  /* forward sweep (:140-188) */
  for (int l = 1; l <= nx - 2; ++l) {
    cplx *g = gl + (size_t)l * b, *gp = gl + (size_t)(l - 1) * b;
    gemm(n, 'N', H10, 'N', gp, Y, w->ta, w->tb);
    gemm(n, 'N', Y, 'C', H10, Z, w->ta, w->tb);
    for (size_t e = 0; e < b; ++e) g[e] = -H0[e] - Z[e];
    for (int i = 0; i < n; ++i) g[i + (size_t)i * n] += z;
    bad |= invert(n, g, w->perm);
    gemm(n, 'N', H10, 'N', gln + (size_t)(l - 1) * b, Y, w->ta, w->tb);
    gemm(n, 'N', Y, 'C', H10, Z, w->ta, w->tb);
    gemm(n, 'N', g, 'N', Z, Y, w->ta, w->tb);
    gemm(n, 'N', Y, 'C', g, gln + (size_t)l * b, w->ta, w->tb);
    gemm(n, 'N', H10, 'N', Pc, Y, w->ta, w->tb);
    gemm(n, 'N', g, 'N', Y, Pc, w->ta, w->tb);
  }
  /* right contact (:192-277) */
  const int N = nx - 1;
  iters[1] = sancho(w, E, eta_lead, tol, nmax, H0, H10, 0, X, &bad);
  gemm(n, 'C', H10, 'N', X, Y, w->ta, w->tb);
  gemm(n, 'N', Y, 'N', H10, SigR, w->ta, w->tb);
  gemm(n, 'N', H10, 'N', gl + (size_t)(N - 1) * b, Y, w->ta, w->tb);
  gemm(n, 'N', Y, 'C', H10, Z, w->ta, w->tb);
  for (size_t e = 0; e < b; ++e) G[e] = -H0[e] - SigR[e] - Z[e];
  for (int i = 0; i < n; ++i) G[i + (size_t)i * n] += z;
  bad |= invert(n, G, w->perm);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      GamR[i + (size_t)j * n] = -(SigR[i + (size_t)j * n] - conj(SigR[j + (size_t)i * n]));
  gemm(n, 'N', H10, 'N', gln + (size_t)(N - 1) * b, Y, w->ta, w->tb);
  gemm(n, 'N', Y, 'C', H10, Z, w->ta, w->tb);
  for (size_t e = 0; e < b; ++e) Z[e] += GamR[e] * fr;
  gemm(n, 'N', G, 'N', Z, Y, w->ta, w->tb);
  gemm(n, 'N', Y, 'C', G, Gn, w->ta, w->tb);
  /* tr = -Re Tr[Gam'_R f G^> - Gam'_R (f-1) G^<] */
  {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        V[i + (size_t)j * n] = Gn[i + (size_t)j * n] + G[i + (size_t)j * n] - conj(G[j + (size_t)i * n]);
    *tr = -(fr * trace_prod(n, GamR, V) - (fr - 1.0) * trace_prod(n, GamR, Gn));
  }
  /* Caroli: G_N1 = G_NN H10 P_{N-1} ; T = -Re Tr[Gam'_R G_N1 Gam'_L G_N1^+] */
  gemm(n, 'N', H10, 'N', Pc, Y, w->ta, w->tb);
  gemm(n, 'N', G, 'N', Y, X, w->ta, w->tb);
  gemm(n, 'N', GamL, 'C', X, Y, w->ta, w->tb);
  gemm(n, 'N', X, 'N', Y, Z, w->ta, w->tb);
  *T = -trace_prod(n, GamR, Z);
  for (int i = 0; i < n; ++i) {
    dgr[(size_t)N * n + i] = G[i + (size_t)i * n];
    dgl[(size_t)N * n + i] = Gn[i + (size_t)i * n];
  }
  /* backward sweep (:283-381), minimal form */
  for (int l = N - 1; l >= 0; --l) {
    const cplx *g = gl + (size_t)l * b, *gn = gln + (size_t)l * b;
    gemm(n, 'N', g, 'C', H10, X, w->ta, w->tb);           /* X = g H^+ */
    gemm(n, 'N', X, 'N', G, Y, w->ta, w->tb);             /* GN0 */
    gemm(n, 'N', H10, 'N', g, Z, w->ta, w->tb);           /* H g */
    gemm(n, 'N', Y, 'N', Z, V, w->ta, w->tb);             /* GN0 H g */
    gemm(n, 'N', X, 'N', Gn, Z, w->ta, w->tb);            /* X G^< */
    gemm(n, 'N', Z, 'C', X, U, w->ta, w->tb);             /* X G^< X^+ */
    for (size_t e = 0; e < b; ++e) G[e] = g[e] + V[e];
    gemm(n, 'N', Y, 'N', H10, Z, w->ta, w->tb);           /* GN0 H */
    gemm(n, 'N', Z, 'N', gn, V, w->ta, w->tb);            /* W */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        Gn[i + (size_t)j * n] = gn[i + (size_t)j * n] + U[i + (size_t)j * n] + V[i + (size_t)j * n] -
                                conj(V[j + (size_t)i * n]);
    for (int i = 0; i < n; ++i) {
      dgr[(size_t)l * n + i] = G[i + (size_t)i * n];
      dgl[(size_t)l * n + i] = Gn[i + (size_t)i * n];
    }
  }
  /* tre (:387-407) */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      V[i + (size_t)j * n] = Gn[i + (size_t)j * n] + G[i + (size_t)j * n] - conj(G[j + (size_t)i * n]);
  *tre = fe * trace_prod(n, GamL, V) - (fe - 1.0) * trace_prod(n, GamL, Gn);
  *status = bad;
}

/* Batched entry point: points p = ie*nk + ik; H00 [nk][nm*nm], H10 [nm*nm] complex128
 * column-major; outputs may be NULL.  Returns the number of points with a status flag. */
int qt_ref_rgf(int nm, int nx, int nk, const double* H00, const double* H10, int nE,
               const double* E, double eta_lead, double eta_int, double tol, int nmax, double mul,
               double mur, double templ, double tempr, int nthreads, double* T, double* tr,
               double* tre, double* dgr, double* dgl, int* status) {
  if (nm <= 0 || nm > 512) return -1;  /* the block product's column buffers hold 512 rows */
  const long long npts = (long long)nE * nk;
  const size_t b = (size_t)nm * nm;
  int nbad = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : nbad)
  {
    Work w;
    work_init(&w, nm);
    cplx* gl = malloc(sizeof(cplx) * b * nx);
    cplx* gln = malloc(sizeof(cplx) * b * nx);
    cplx* s = malloc(sizeof(cplx) * b * 12);
    cplx* dr = malloc(sizeof(cplx) * (size_t)nm * nx);
    cplx* dl = malloc(sizeof(cplx) * (size_t)nm * nx);
#pragma omp for schedule(dynamic, 1)
    for (long long p = 0; p < npts; ++p) {
      const int ie = (int)(p / nk), ik = (int)(p % nk);
      const double e = E[ie];
      const double fl = ferm((e - mul) / (BOLTZ * templ));
      const double fr = ferm((e - mur) / (BOLTZ * templ));
      const double fe = ferm((e - mul) / (BOLTZ * tempr));
      double t, a, c;
      int st, it[2];
      point(&w, nx, e, (const cplx*)H00 + (size_t)ik * b, (const cplx*)H10, eta_lead, eta_int, tol,
            nmax, fl, fr, fe, gl, gln, s, &t, &a, &c, dr, dl, &st, it);
      if (T) T[p] = t;
      if (tr) tr[p] = a;
      if (tre) tre[p] = c;
      if (dgr) memcpy(dgr + 2 * (size_t)p * nx * nm, dr, sizeof(cplx) * nx * nm);
      if (dgl) memcpy(dgl + 2 * (size_t)p * nx * nm, dl, sizeof(cplx) * nx * nm);
      if (status) status[p] = st;
      nbad += st != 0;
    }
    free(gl); free(gln); free(s); free(dr); free(dl);
    work_free(&w);
  }
  return nbad;
}
