/*
 * CPU restatement of the reference RGF sweep -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain C99 + OpenMP (parallel over independent (E, k) points), complex128,
 * column-major n x n blocks.  It follows, step for step:
 *   sancho                    src/cuda_rgf_mod.f90:657-765 (src/rgf_mod.f90:482-568)
 *   cuda_rgf_constblocksize   src/cuda_rgf_mod.f90:53-413, with G^> = G^< + G - G^+
 *                             in every slab (what produced test_cnt/pdos0000.dat)
 * plus the Caroli transmission Tr[Gam_R G_N1 Gam_L G_N1^+].  Block products run on
 * packed real / imaginary planes with register-blocked tiles of C, and inverses
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

/* C = op(A) op(B)  (op: 'N' or 'C'), all n x n column-major.  The operands are first packed
 * into real and imaginary planes with op applied: op(A) in panels of MR rows stored
 * [panel][k][MR], op(B) in panels of NR columns stored [panel][k][NR], zero-padded past n.
 * Each MR x NR tile of C then accumulates in registers (two-double vectors of GCC's
 * generic vector extension, the same on every target), every loaded pair of a panel
 * feeding NR complex multiply-adds, so the loop is bound by multiply-adds rather than by
 * loads and stores.  Every C(i, j) accumulates over k = 0 .. n-1 in order with the same
 * expression as an unblocked loop.  The tile is 4 x 4 where 32 vector registers hold it
 * (aarch64) and 4 x 2 elsewhere.  ta, tb hold (n + 4) n complex each. */
typedef double v2d __attribute__((vector_size(16)));
#if defined(__aarch64__)
enum { MR = 4, NR = 4 };
#else
enum { MR = 4, NR = 2 };
#endif
static inline v2d ld2(const double* p) {
  v2d v;
  memcpy(&v, p, sizeof v);
  return v;
}
static void gemm(int n, char opa, const cplx* A, char opb, const cplx* B, cplx* C, cplx* ta,
                 cplx* tb) {
  const int pi = (n + MR - 1) / MR, pj = (n + NR - 1) / NR;
  double* restrict ar = (double*)ta;
  double* restrict ai = ar + (size_t)pi * n * MR;
  double* restrict br = (double*)tb;
  double* restrict bi = br + (size_t)pj * n * NR;
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < pi * MR; ++i) {
      const cplx x = i >= n ? 0.0 : opa == 'C' ? conj(A[k + (size_t)i * n]) : A[i + (size_t)k * n];
      const size_t o = ((size_t)(i / MR) * n + k) * MR + i % MR;
      ar[o] = creal(x);
      ai[o] = cimag(x);
    }
  for (int j = 0; j < pj * NR; ++j)
    for (int k = 0; k < n; ++k) {
      const cplx y = j >= n ? 0.0 : opb == 'C' ? conj(B[j + (size_t)k * n]) : B[k + (size_t)j * n];
      const size_t o = ((size_t)(j / NR) * n + k) * NR + j % NR;
      br[o] = creal(y);
      bi[o] = cimag(y);
    }
  for (int jp = 0; jp < pj; ++jp)
    for (int ip = 0; ip < pi; ++ip) {
      const double* restrict xr = ar + (size_t)ip * n * MR;
      const double* restrict xi = ai + (size_t)ip * n * MR;
      const double* restrict yr = br + (size_t)jp * n * NR;
      const double* restrict yi = bi + (size_t)jp * n * NR;
      v2d cr[NR][MR / 2], ci[NR][MR / 2];
      for (int q = 0; q < NR; ++q)
        for (int h = 0; h < MR / 2; ++h) cr[q][h] = ci[q][h] = (v2d){0.0, 0.0};
      for (int k = 0; k < n; ++k) {
        v2d pr[MR / 2], pm[MR / 2];
        for (int h = 0; h < MR / 2; ++h) {
          pr[h] = ld2(xr + (size_t)k * MR + 2 * h);
          pm[h] = ld2(xi + (size_t)k * MR + 2 * h);
        }
        for (int q = 0; q < NR; ++q) {
          const double wr = yr[(size_t)k * NR + q], wi = yi[(size_t)k * NR + q];
          const v2d vr = {wr, wr}, vi = {wi, wi};
          for (int h = 0; h < MR / 2; ++h) {
            cr[q][h] += pr[h] * vr - pm[h] * vi;
            ci[q][h] += pr[h] * vi + pm[h] * vr;
          }
        }
      }
      for (int q = 0; q < NR; ++q) {
        const int j = jp * NR + q;
        if (j >= n) break;
        for (int r = 0; r < MR; ++r) {
          const int i = ip * MR + r;
          if (i < n) C[i + (size_t)j * n] = cr[q][r / 2][r % 2] + I * ci[q][r / 2][r % 2];
        }
      }
    }
}

/* in-place inverse, Gauss-Jordan with row pivoting (|re|+|im| pivot measure).  The
 * elimination runs on real and imaginary planes (xr: 2 n^2 doubles of scratch), so the
 * rank-1 update of each column is a loop of real multiply-adds that vectorises; every
 * element sees the same complex operations as on interleaved storage. */
static int invert(int n, cplx* X, int* perm, double* restrict xr) {
  const size_t nn = (size_t)n * n;
  double* restrict xi = xr + nn;
  for (size_t e = 0; e < nn; ++e) {
    xr[e] = creal(X[e]);
    xi[e] = cimag(X[e]);
  }
  int bad = 0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1.0;
    for (int i = k; i < n; ++i) {
      const double m = fabs(xr[i + (size_t)k * n]) + fabs(xi[i + (size_t)k * n]);
      if (m > best) { best = m; p = i; }
    }
    if (!(best > 0.0)) bad = 1;
    perm[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) {
        const size_t a = k + (size_t)j * n, b = p + (size_t)j * n;
        const double tr = xr[a], ti = xi[a];
        xr[a] = xr[b]; xi[a] = xi[b];
        xr[b] = tr; xi[b] = ti;
      }
    const cplx piv = xr[k + (size_t)k * n] + I * xi[k + (size_t)k * n];
    const cplx inv = best > 0.0 ? 1.0 / piv : 0.0;
    const double vr = creal(inv), vi = cimag(inv);
    for (int j = 0; j < n; ++j) {
      const size_t a = k + (size_t)j * n;
      const double u = xr[a], v = xi[a];
      xr[a] = u * vr - v * vi;
      xi[a] = u * vi + v * vr;
    }
    xr[k + (size_t)k * n] = vr;
    xi[k + (size_t)k * n] = vi;
    const double* restrict ckr = xr + (size_t)k * n;
    const double* restrict cki = xi + (size_t)k * n;
    for (int j = 0; j < n; ++j) {
      if (j == k) continue;
      const double rr = xr[k + (size_t)j * n], ri = xi[k + (size_t)j * n];
      double* restrict cr = xr + (size_t)j * n;
      double* restrict ci = xi + (size_t)j * n;
      /* all rows, then row k put back: the same operations on rows i != k, in a loop
         without a branch */
      for (int i = 0; i < n; ++i) {
        cr[i] -= ckr[i] * rr - cki[i] * ri;
        ci[i] -= ckr[i] * ri + cki[i] * rr;
      }
      cr[k] = rr;
      ci[k] = ri;
    }
    const double nr = -vr, ni = -vi;
    for (int i = 0; i < n; ++i)
      if (i != k) {
        const size_t a = i + (size_t)k * n;
        const double u = xr[a], v = xi[a];
        xr[a] = u * nr - v * ni;
        xi[a] = u * ni + v * nr;
      }
  }
  for (size_t e = 0; e < nn; ++e) X[e] = xr[e] + I * xi[e];
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
  const size_t b = (size_t)n * n, t = b + 4 * (size_t)n;  /* packed panels, padded to 4 */
  w->n = n;
  w->A = malloc(sizeof(cplx) * (b * 8 + 2 * t));
  w->B = w->A + b; w->C = w->B + b; w->D = w->C + b; w->ta = w->D + b; w->tb = w->ta + t;
  w->HBB = w->tb + t; w->HSS = w->HBB + b; w->H10 = w->HSS + b; w->H01 = w->H10 + b;
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
    *bad |= invert(n, w->A, w->perm, (double*)w->ta);
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
  *bad |= invert(n, G00, w->perm, (double*)w->ta);
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
  bad |= invert(n, gl, w->perm, (double*)w->ta);
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
    bad |= invert(n, g, w->perm, (double*)w->ta);
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
  bad |= invert(n, G, w->perm, (double*)w->ta);
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
  if (nm <= 0) return -1;
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
