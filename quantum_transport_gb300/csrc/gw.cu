// GW/SCBA self-energy loop on the GPU (rows of gw_ephoton_3d_ijs,
// src/gw_mod.f90:444-749).
//
// Data layout: every energy-resolved quantity (G^{R,<,>}, P, W, Sigma) is an
// array [nk][nE][nx][nm*nm] of complex128 column-major slab-diagonal blocks, k
// slowest as in the reference's (nm, nm, nx, nE, nk) arrays; per k-point it is the
// block layout qt_rgf_solve reads (sigmas) and writes (full G blocks).  An energy
// SERIES is one matrix element (i, j) of one slab at one k followed through the
// energy grid: element stride nx*nm*nm.  With several k-points the polarisation
// and self-energy sum over k-pairs (src/gw_mod.f90:476-512, 653-690), and the
// ndiag band skips the elements |i - j| > ndiag (:471-475).
//
//  * zcorrconv: batched energy correlation / convolution through zero-padded
//    radix-2 FFTs in shared memory (one CTA per series, L = 2^ceil(log2 2n)),
//    replacing corr1d2 / conv1d2 + MKL DFTI (src/fft_mod.f90:58-190), which
//    created a new DFTI descriptor for every series:
//      corr(X, Y)[m] = sum_e X[e] Y[e - (m - n/2)]
//      conv(X, W)[e] = sum_m X[e - (m - n/2)] W[m]
//    FP64 arithmetic: the SCBA residual target (1e-8) is below FP32 resolution.
//  * sigma_post: Sigma^R <- Re Sigma^R + i Im(Sigma^> - Sigma^<)/2 and the
//    symmetrisation (Sigma + Sigma^T)/2 (src/gw_mod.f90:698, 731-743).
//  * mix_residual: linear mixing (:747-749) with the residual norms.
#include <cmath>

#include "qt_common.cuh"
#include "qt_kernels.h"

namespace qt {

namespace {

constexpr int FFT_NT = 256;
constexpr int LMAX = 4096;

__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void twiddle_kernel(double2* tw) {
  // tw[k] = exp(-2 pi i k / LMAX), k < LMAX/2
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < LMAX / 2; k += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * k / LMAX, &s, &c);
    tw[k] = make_double2(c, s);
  }
}

__device__ __forceinline__ void butterfly(double2& u, double2& v, double2 w) {
  const double2 x = u, y = dmul(v, w);
  u = make_double2(x.x + y.x, x.y + y.y);
  v = make_double2(x.x - y.x, x.y - y.y);
}

// twiddle tw[j], conjugated for the inverse transform (the sign folds into the FMAs)
template <bool INV>
__device__ __forceinline__ double2 twiddle(const double2* tw, int j) {
  const double2 w = tw[j];
  return INV ? make_double2(w.x, -w.y) : w;
}

// u, v <- u + v, u - v: a butterfly whose twiddle is exactly 1
__device__ __forceinline__ void butterfly1(double2& u, double2& v) {
  const double2 x = u, y = v;
  u = make_double2(x.x + y.x, x.y + y.y);
  v = make_double2(x.x - y.x, x.y - y.y);
}

// u, v <- u + r y, u - r y with r = -i (forward) or +i (inverse) and y = v w already formed:
// tw[j + LMAX/4] = tw[j] (-i), so the second twiddle of a radix-4 pair is a rotation of the
// first and costs no multiply
template <bool INV>
__device__ __forceinline__ void butterfly_rot(double2& u, double2& v, double2 y) {
  const double2 x = u;
  const double2 r = INV ? make_double2(-y.y, y.x) : make_double2(y.y, -y.x);
  u = make_double2(x.x + r.x, x.y + r.y);
  v = make_double2(x.x - r.x, x.y - r.y);
}

// In-place iterative radix-2 DIT on bit-reversed input; exponent sign -1 forward (INV
// false), +1 inverse.  Stages go through shared memory in pairs: a thread takes the four elements
// base + {0, h, 2h, 3h} of a 4h-block, applies stage s to (0, h) and (2h, 3h) and stage s+1
// to (0, 2h) and (h, 3h) in registers -- the butterflies of two radix-2 passes with half the
// shared-memory passes and barriers.  Stage s+1's twiddle for (h, 3h) is that of (0, 2h)
// times -i (+i inverse), applied as a rotation; the first pair's twiddles are 1 and -i, so
// it has no multiplies.  An odd stage count starts with one single radix-2 pass (twiddle 1).
template <bool INV>
__device__ __forceinline__ void fft_smem(double2* a, int L, int logL, const double2* tw) {
  int s = 1;
  if (logL & 1) {
    for (int t = threadIdx.x; t < L / 2; t += blockDim.x) butterfly1(a[2 * t], a[2 * t + 1]);
    __syncthreads();
    s = 2;
  }
  for (; s < logL; s += 2) {
    const int h = 1 << (s - 1);
    const int step1 = LMAX / (2 * h), step2 = LMAX / (4 * h);
    for (int t = threadIdx.x; t < L / 4; t += blockDim.x) {
      const int grp = t >> (s - 1), k = t & (h - 1);
      const int b = grp * 4 * h + k;
      double2 e0 = a[b], e1 = a[b + h], e2 = a[b + 2 * h], e3 = a[b + 3 * h];
      if (h == 1) {  // k = 0: twiddles 1, 1 and -i (+i); uniform over the block
        butterfly1(e0, e1);
        butterfly1(e2, e3);
        butterfly1(e0, e2);
        butterfly_rot<INV>(e1, e3, e3);
      } else {
        const double2 v1 = twiddle<INV>(tw, k * step1), v2 = twiddle<INV>(tw, k * step2);
        butterfly(e0, e1, v1);  // stage s
        butterfly(e2, e3, v1);
        butterfly(e0, e2, v2);  // stage s + 1
        butterfly_rot<INV>(e1, e3, dmul(e3, v2));
      }
      a[b] = e0;
      a[b + h] = e1;
      a[b + 2 * h] = e2;
      a[b + 3 * h] = e3;
    }
    __syncthreads();
  }
}

// load one series pair into bit-reversed shared-memory buffers x, y (zero-padded to L)
__device__ __forceinline__ void load_pair(const CorrConvArgs& a, const double2* X,
                                          const double2* Y, const double2* Yb, long long sx,
                                          long long sy, int conjY, double2* x, double2* y) {
  const int n = a.n, L = a.L, logL = a.logL;
  for (int t = threadIdx.x; t < L; t += blockDim.x) {
    double2 vx = make_double2(0.0, 0.0), vy = vx;
    if (t < n) {
      vx = X[(long long)t * a.estride + sx];
      if (a.imagX) vx.x = 0.0;
      const int ty = a.corr ? (n - 1 - t) : t;  // correlation: reversed Y
      vy = Y[(long long)ty * a.estride + sy];
      if (Yb) {
        const double2 b = Yb[(long long)ty * a.estride + sy];
        vy.x += b.x;
        vy.y += b.y;
      }
      if (a.imagY) vy.x = 0.0;
      if (conjY) vy.y = -vy.y;
    }
    const int r = (int)(__brev((unsigned)t) >> (32 - logL));
    x[r] = vx;
    y[r] = vy;
  }
}

// 0-based k-pair partner of ik and iq: per direction kd = k - q + nk_dir/2 (1-based
// indices, integer division) wrapped once into range (src/gw_mod.f90:478-487, 658-667)
__device__ __forceinline__ int kpair(int ik, int iq, int nky, int nkz) {
  const int iky = ik / nkz, ikz = ik - iky * nkz, iqy = iq / nkz, iqz = iq - iqy * nkz;
  int kzd = (ikz - iqz + nkz / 2 - 1) % nkz;
  int kyd = (iky - iqy + nky / 2 - 1) % nky;
  if (kzd < 0) kzd += nkz;
  if (kyd < 0) kyd += nky;
  return kzd + kyd * nkz;
}

// One output series per CTA iteration: for each k-pair (one with kmode 0) and term, the
// two series are loaded bit-reversed into b1, b2, transformed, and their product summed
// into acc (b1 itself when there is one product only); then one inverse transform.
__global__ void __launch_bounds__(FFT_NT, 1) zcorrconv_kernel(CorrConvArgs a, const double2* tw) {
  extern __shared__ double2 sm[];
  const int n = a.n, L = a.L, logL = a.logL, nk = a.nk;
  const bool two = a.X2 != nullptr;
  const int tn = a.kmode ? nk : 1;
  double2* b1 = sm;
  double2* b2 = sm + L;
  double2* acc = (two || tn > 1) ? sm + 2 * L : b1;
  double2* inv_buf = acc == b1 ? b2 : b1;
  const long long nm2 = (long long)a.nm * a.nm, nel = a.nel ? a.nel : nm2;
  const double2* X = reinterpret_cast<const double2*>(a.X);
  const double2* Y = reinterpret_cast<const double2*>(a.Y);
  const double2* X2 = reinterpret_cast<const double2*>(a.X2);
  const double2* Y2 = reinterpret_cast<const double2*>(a.Y2);
  const double2* Y2b = reinterpret_cast<const double2*>(a.Y2b);
  double2* Z = reinterpret_cast<double2*>(a.Z);
  const long long total = (long long)nk * a.nseries;
  for (long long s = blockIdx.x; s < total; s += gridDim.x) {
    const int o = (int)(s / a.nseries);
    const long long r = s - (long long)o * a.nseries;
    const long long ix = r / nel, el = r - ix * nel, ij = a.ij0 + el;
    const int i = (int)(ij % a.nm), j = (int)(ij / a.nm);
    const long long rt = ix * nel + i * (long long)a.nm + j;  // the transposed element
    double2* Zo = Z + o * a.kstride;
    if (a.ndiag >= 0 && abs(i - j) > a.ndiag) {  // outside the band: the series is zero
      if (!a.accumulate)
        for (int m = threadIdx.x; m < n; m += blockDim.x)
          Zo[(long long)m * a.estride + r] = make_double2(0.0, 0.0);
      continue;  // uniform over the CTA
    }
    for (int t = 0; t < tn; ++t) {
      int xs = o, ys = o;
      if (a.kmode == 1) { xs = t; ys = kpair(t, o, a.nky, a.nkz); }
      else if (a.kmode == 2) { xs = kpair(o, t, a.nky, a.nkz); ys = t; }
      for (int term = 0; term < (two ? 2 : 1); ++term) {
        const long long xo = xs * a.kstride, yo = ys * a.kstride;
        if (term == 0)
          load_pair(a, X + xo, Y + yo, nullptr, r, a.transY ? rt : r, a.conjY, b1, b2);
        else
          load_pair(a, X2 + xo, Y2 + yo, Y2b ? Y2b + yo : nullptr, r, a.transY2 ? rt : r,
                    a.conjY2, b1, b2);
        __syncthreads();
        fft_smem<false>(b1, L, logL, tw);
        fft_smem<false>(b2, L, logL, tw);
        const bool first = t == 0 && term == 0;
        for (int q = threadIdx.x; q < L; q += blockDim.x) {
          const double2 p = dmul(b1[q], b2[q]);
          acc[q] = first ? p : make_double2(acc[q].x + p.x, acc[q].y + p.y);
        }
        __syncthreads();
      }
    }
    // bit-reversed into the free buffer for the inverse transform
    for (int q = threadIdx.x; q < L; q += blockDim.x)
      inv_buf[(int)(__brev((unsigned)q) >> (32 - logL))] = acc[q];
    __syncthreads();
    fft_smem<true>(inv_buf, L, logL, tw);
    const double inv = 1.0 / L;
    const double2 sc = make_double2(a.scale_re * inv, a.scale_im * inv);
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
      const int q = a.corr ? (m - n / 2 + n - 1) : (m + n / 2);
      const double2 v = dmul(inv_buf[q], sc);
      double2* zp = &Zo[(long long)m * a.estride + r];
      if (a.accumulate) {
        const double2 w = *zp;
        *zp = make_double2(w.x + v.x, w.y + v.y);
      } else {
        *zp = v;
      }
    }
    __syncthreads();
  }
}

// ---- packed transforms of purely imaginary series (one k-point)
__device__ __forceinline__ double2 dconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 dscale(double2 a, double c) { return make_double2(c * a.x, c * a.y); }
__device__ __forceinline__ double2 times_i(double2 a) { return make_double2(-a.y, a.x); }

// the transforms of the real sequences a, b packed as z = a + i b: from Z(k) and Z(L - k),
// A(k) = (Z(k) + conj Z(L-k))/2, B(k) = (Z(k) - conj Z(L-k))/(2i)
__device__ __forceinline__ void unpack(double2 zk, double2 zkk, double2& A, double2& B) {
  const double2 q = dconj(zkk);
  A = dscale(dadd(zk, q), 0.5);
  const double2 d = dscale(dsub(zk, q), 0.5);
  B = make_double2(d.y, -d.x);  // d / i
}

// in-place bit-reversal permutation (natural order -> the FFT's bit-reversed input)
__device__ __forceinline__ void bitrev_permute(double2* a, int L, int logL) {
  for (int t = threadIdx.x; t < L; t += blockDim.x) {
    const int r = (int)(__brev((unsigned)t) >> (32 - logL));
    if (t < r) {
      const double2 x = a[t];
      a[t] = a[r];
      a[r] = x;
    }
  }
}

// element (series r, partner rt) of one energy series; false outside the band
__device__ __forceinline__ bool series_of(const GwFusedArgs& a, long long r, long long& rt) {
  const long long nm2 = (long long)a.nm * a.nm, nel = a.nel ? a.nel : nm2;
  const long long ix = r / nel, el = r - ix * nel, ij = a.ij0 + el;
  const int i = (int)(ij % a.nm), j = (int)(ij / a.nm);
  rt = ix * nel + i * (long long)a.nm + j;
  return a.ndiag < 0 || abs(i - j) <= a.ndiag;
}

// P^<, P^>, P^R of one series per CTA: three packed forward transforms
// (G^<, G^>), (rev G^>t, rev G^<t), (G^R, rev conj G^R) of the imaginary parts, the three
// products per frequency, three inverse transforms.  Each product of two imaginary series'
// transforms is -A B of their imaginary parts' transforms.
__global__ void __launch_bounds__(FFT_NT, 1) gw_pol_kernel(GwFusedArgs a, const double2* tw) {
  extern __shared__ double2 sm[];
  const int n = a.n, L = a.L, logL = a.logL;
  double2 *b0 = sm, *b1 = sm + L, *b2 = sm + 2 * L;
  const double2* GR = reinterpret_cast<const double2*>(a.GR);
  const double2* GL = reinterpret_cast<const double2*>(a.GL);
  const double2* GG = reinterpret_cast<const double2*>(a.GG);
  const double2* GLt = reinterpret_cast<const double2*>(a.GLt ? a.GLt : a.GL);
  const double2* GGt = reinterpret_cast<const double2*>(a.GGt ? a.GGt : a.GG);
  double2* P[3] = {reinterpret_cast<double2*>(a.PL), reinterpret_cast<double2*>(a.PG),
                   reinterpret_cast<double2*>(a.PR)};
  const long long es = a.estride;
  const double inv = 1.0 / L;
  const double2 sc = make_double2(a.scale_re * inv, a.scale_im * inv);
  for (long long r = blockIdx.x; r < a.nseries; r += gridDim.x) {
    long long rt;
    if (!series_of(a, r, rt)) {
      for (int m = threadIdx.x; m < n; m += blockDim.x)
        for (int q = 0; q < 3; ++q) P[q][(long long)m * es + r] = make_double2(0.0, 0.0);
      continue;  // uniform over the CTA
    }
    const long long rp = a.GLt ? r : rt;  // where the transposed partner is stored
    for (int t = threadIdx.x; t < L; t += blockDim.x) {
      const int p = (int)(__brev((unsigned)t) >> (32 - logL));
      double2 z0 = make_double2(0.0, 0.0), z1 = z0, z2 = z0;
      if (t < n) {
        const long long f = (long long)t * es, bk = (long long)(n - 1 - t) * es;
        z0 = make_double2(GL[f + r].y, GG[f + r].y);
        z1 = make_double2(GGt[bk + rp].y, GLt[bk + rp].y);
        z2 = make_double2(GR[f + r].y, -GR[bk + r].y);  // Im conj G^R(n-1-t) = -Im G^R(n-1-t)
      }
      b0[p] = z0;
      b1[p] = z1;
      b2[p] = z2;
    }
    __syncthreads();
    fft_smem<false>(b0, L, logL, tw);
    fft_smem<false>(b1, L, logL, tw);
    fft_smem<false>(b2, L, logL, tw);
    for (int k = threadIdx.x; k <= L / 2; k += blockDim.x) {
      const int kk = (L - k) & (L - 1);
      double2 A1, B1, A2, B2, A3, B3;
      unpack(b0[k], b0[kk], A1, B1);
      unpack(b1[k], b1[kk], A2, B2);
      unpack(b2[k], b2[kk], A3, B3);
      const double2 pl = dscale(dmul(A1, A2), -1.0);
      const double2 pg = dscale(dmul(B1, B2), -1.0);
      const double2 pr = dscale(dadd(dmul(A1, B3), dmul(A3, B2)), -1.0);
      b0[k] = pl; b1[k] = pg; b2[k] = pr;
      if (kk != k) {  // the transforms of real sequences' products: Hermitian
        b0[kk] = dconj(pl); b1[kk] = dconj(pg); b2[kk] = dconj(pr);
      }
    }
    __syncthreads();
    bitrev_permute(b0, L, logL);
    bitrev_permute(b1, L, logL);
    bitrev_permute(b2, L, logL);
    __syncthreads();
    fft_smem<true>(b0, L, logL, tw);
    fft_smem<true>(b1, L, logL, tw);
    fft_smem<true>(b2, L, logL, tw);
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
      const int q = m - n / 2 + n - 1;
      P[0][(long long)m * es + r] = dmul(b0[q], sc);
      P[1][(long long)m * es + r] = dmul(b1[q], sc);
      P[2][(long long)m * es + r] = dmul(b2[q], sc);
    }
    __syncthreads();
  }
}

// Sigma^>, then Sigma^< and Sigma^R, of one series per CTA.  Phase 1: transforms of i Im G^>
// and W^>, product, inverse.  Phase 2: the packed transform of (Im G^<, Im G^R) and the
// transforms of W^<, W^R; per frequency S^< = i A W^<, S^R = i A W^R + i B (W^< + W^R);
// two inverses.  The outputs may overwrite G: every read of the series precedes its writes.
__global__ void __launch_bounds__(FFT_NT, 1) gw_sig_kernel(GwFusedArgs a, const double2* tw) {
  extern __shared__ double2 sm[];
  const int n = a.n, L = a.L, logL = a.logL;
  double2 *b0 = sm, *b1 = sm + L, *b2 = sm + 2 * L;
  const double2* GR = reinterpret_cast<const double2*>(a.GR);
  const double2* GL = reinterpret_cast<const double2*>(a.GL);
  const double2* GG = reinterpret_cast<const double2*>(a.GG);
  const double2* WR = reinterpret_cast<const double2*>(a.WR);
  const double2* WL = reinterpret_cast<const double2*>(a.WL);
  const double2* WG = reinterpret_cast<const double2*>(a.WG);
  double2* SR = reinterpret_cast<double2*>(a.SR);
  double2* SL = reinterpret_cast<double2*>(a.SL);
  double2* SG = reinterpret_cast<double2*>(a.SG);
  const long long es = a.estride;
  const double inv = 1.0 / L;
  const double2 sc = make_double2(a.scale_re * inv, a.scale_im * inv);
  for (long long r = blockIdx.x; r < a.nseries; r += gridDim.x) {
    long long rt;
    if (!series_of(a, r, rt)) {
      for (int m = threadIdx.x; m < n; m += blockDim.x) {
        const long long o = (long long)m * es + r;
        SR[o] = make_double2(0.0, 0.0);
        SL[o] = make_double2(0.0, 0.0);
        SG[o] = make_double2(0.0, 0.0);
      }
      continue;
    }
    // phase 1: Sigma^> = s conv(i Im G^>, W^>)
    for (int t = threadIdx.x; t < L; t += blockDim.x) {
      const int p = (int)(__brev((unsigned)t) >> (32 - logL));
      double2 x = make_double2(0.0, 0.0), w = x;
      if (t < n) {
        const long long f = (long long)t * es + r;
        x = make_double2(0.0, GG[f].y);
        w = WG[f];
      }
      b0[p] = x;
      b1[p] = w;
    }
    __syncthreads();
    fft_smem<false>(b0, L, logL, tw);
    fft_smem<false>(b1, L, logL, tw);
    for (int k = threadIdx.x; k < L; k += blockDim.x) b0[k] = dmul(b0[k], b1[k]);
    __syncthreads();
    bitrev_permute(b0, L, logL);
    __syncthreads();
    fft_smem<true>(b0, L, logL, tw);
    for (int m = threadIdx.x; m < n; m += blockDim.x)
      SG[(long long)m * es + r] = dmul(b0[m + n / 2], sc);
    __syncthreads();
    // phase 2: Sigma^< and Sigma^R
    for (int t = threadIdx.x; t < L; t += blockDim.x) {
      const int p = (int)(__brev((unsigned)t) >> (32 - logL));
      double2 z = make_double2(0.0, 0.0), wl = z, wr = z;
      if (t < n) {
        const long long f = (long long)t * es + r;
        z = make_double2(GL[f].y, GR[f].y);
        wl = WL[f];
        wr = WR[f];
      }
      b0[p] = z;
      b1[p] = wl;
      b2[p] = wr;
    }
    __syncthreads();
    fft_smem<false>(b0, L, logL, tw);
    fft_smem<false>(b1, L, logL, tw);
    fft_smem<false>(b2, L, logL, tw);
    for (int k = threadIdx.x; k <= L / 2; k += blockDim.x) {
      const int kk = (L - k) & (L - 1);
      double2 A, B;
      unpack(b0[k], b0[kk], A, B);  // transforms of Im G^< and Im G^R at k
      const double2 wlk = b1[k], wrk = b2[k], wlkk = b1[kk], wrkk = b2[kk];
      b1[k] = times_i(dmul(A, wlk));
      b2[k] = times_i(dadd(dmul(A, wrk), dmul(B, dadd(wlk, wrk))));
      if (kk != k) {
        const double2 Ak = dconj(A), Bk = dconj(B);  // the transforms at L - k
        b1[kk] = times_i(dmul(Ak, wlkk));
        b2[kk] = times_i(dadd(dmul(Ak, wrkk), dmul(Bk, dadd(wlkk, wrkk))));
      }
    }
    __syncthreads();
    bitrev_permute(b1, L, logL);
    bitrev_permute(b2, L, logL);
    __syncthreads();
    fft_smem<true>(b1, L, logL, tw);
    fft_smem<true>(b2, L, logL, tw);
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
      const long long o = (long long)m * es + r;
      SL[o] = dmul(b1[m + n / 2], sc);
      SR[o] = dmul(b2[m + n / 2], sc);
    }
    __syncthreads();
  }
}

// zero |i - j| > ndiag of column-major nm x nm blocks bstride elements apart
// (src/gw_mod.f90:527-555, 705-730)
__global__ void band_zero_kernel(int nm, long long count, long long bstride, int ndiag,
                                 double2* A) {
  const long long nm2 = (long long)nm * nm;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / nm2, e = t - b * nm2;
    const int i = (int)(e % nm), j = (int)(e / nm);
    if (abs(i - j) > ndiag) A[b * bstride + e] = make_double2(0.0, 0.0);
  }
}

// Sigma^R <- Re Sigma^R + i Im(Sigma^> - Sigma^<)/2, then (S + S^T)/2 for all three,
// one CTA per (energy, slab) block (src/gw_mod.f90:698, 731-743)
__global__ void sigma_post_kernel(int nm, long long nblocks, double2* SR, double2* SL,
                                  double2* SG) {
  const long long nm2 = (long long)nm * nm;
  for (long long b = blockIdx.x; b < nblocks; b += gridDim.x) {
    double2 *r = SR + b * nm2, *l = SL + b * nm2, *g = SG + b * nm2;
    for (int e = threadIdx.x; e < nm * nm; e += blockDim.x) {
      const int i = e % nm, j = e / nm;
      if (i > j) continue;  // the thread owning (i<=j) writes both (i,j) and (j,i)
      const long long a1 = i + (long long)j * nm, a2 = j + (long long)i * nm;
      const double2 r1 = r[a1], r2 = r[a2], l1 = l[a1], l2 = l[a2], g1 = g[a1], g2 = g[a2];
      const double2 rr1 = make_double2(r1.x, 0.5 * (g1.y - l1.y));
      const double2 rr2 = make_double2(r2.x, 0.5 * (g2.y - l2.y));
      const double2 rs = make_double2(0.5 * (rr1.x + rr2.x), 0.5 * (rr1.y + rr2.y));
      const double2 ls = make_double2(0.5 * (l1.x + l2.x), 0.5 * (l1.y + l2.y));
      const double2 gs = make_double2(0.5 * (g1.x + g2.x), 0.5 * (g1.y + g2.y));
      r[a1] = rs; r[a2] = rs;
      l[a1] = ls; l[a2] = ls;
      g[a1] = gs; g[a2] = gs;
    }
  }
}

// sums[0] += |new - old|^2, sums[1] += |new|^2 over count elements (Sigma^< and Sigma^>)
__global__ void residual_kernel(long long count, const double2* nl, const double2* ol,
                                const double2* ng, const double2* og, double* sums) {
  double d = 0.0, m = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    const double2 a = nl[t], b = ol[t], c = ng[t], e = og[t];
    d += (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (c.x - e.x) * (c.x - e.x) +
         (c.y - e.y) * (c.y - e.y);
    m += a.x * a.x + a.y * a.y + c.x * c.x + c.y * c.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    d += __shfl_down_sync(0xffffffffu, d, o);
    m += __shfl_down_sync(0xffffffffu, m, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&sums[0], d);
    atomicAdd(&sums[1], m);
  }
}

// S <- S + alpha (N - S)   (linear mixing, src/gw_mod.f90:747-749)
__global__ void mix_kernel(long long count, double alpha, double2* S, const double2* N) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    const double2 s = S[t], v = N[t];
    S[t] = make_double2(s.x + alpha * (v.x - s.x), s.y + alpha * (v.y - s.y));
  }
}

// A[e] = scale (G[e - nop] + G[e + nop]) per (energy, slab) block, the photon-shifted sum
// of calc_sigma_ephoton_monochromatic_ext (src/gw_mod.f90:1095-1110), with the
// self-energy's prefactor applied here in FP64 (the split products that follow take
// their alpha in FP32).  With halo != 0, G
// holds nE + 2 nop energies (nop exchanged from each neighbouring energy shard, zero
// beyond the global grid) and energy e of the output reads G[e] + G[e + 2 nop]; without,
// G holds nE energies and terms outside [0, nE) are zero.
__global__ void photon_shift_sum_kernel(long long per, long long nE, int nop, int halo,
                                        double scale, const double2* G, double2* A) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nE * per;
       t += (long long)gridDim.x * blockDim.x) {
    const long long e = t / per, r = t - e * per;
    const long long lo = halo ? e : e - nop, hi = halo ? e + 2 * nop : e + nop;
    const long long ne = halo ? nE + 2 * nop : nE;
    double2 v = make_double2(0.0, 0.0);
    if (lo >= 0) { const double2 a = G[lo * per + r]; v.x += a.x; v.y += a.y; }
    if (hi < ne) { const double2 b = G[hi * per + r]; v.x += b.x; v.y += b.y; }
    A[t] = make_double2(scale * v.x, scale * v.y);
  }
}

// Sigma^R = i Im(Sigma^> - Sigma^<) / 2, real part zero (src/gw_mod.f90:1121)
__global__ void photon_retarded_kernel(long long count, const double2* SL, const double2* SG,
                                       double2* SR) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x)
    SR[t] = make_double2(0.0, 0.5 * (SG[t].y - SL[t].y));
}

inline unsigned g1(long long n) {
  long long g = (n + 255) / 256;
  return (unsigned)(g < 1 ? 1 : (g > 65535LL * 8 ? 65535LL * 8 : g));
}

}  // namespace

cudaError_t gw_twiddles(double2* tw, cudaStream_t s) {
  twiddle_kernel<<<8, 256, 0, s>>>(tw);
  count_launch();
  return cudaGetLastError();
}

cudaError_t zcorrconv(CorrConvArgs a, const double2* tw, cudaStream_t s) {
  if (a.nseries <= 0) return cudaSuccess;
  int L = 1, logL = 0;
  while (L < 2 * a.n) { L <<= 1; ++logL; }
  if (L > LMAX) return cudaErrorInvalidValue;
  a.L = L;
  a.logL = logL;
  if (a.nk < 1 || a.nky * a.nkz != a.nk) return cudaErrorInvalidValue;
  if (a.nk > 1 && a.kmode != 0 &&
      (a.Z == a.X || a.Z == a.Y || (a.X2 && (a.Z == a.X2 || a.Z == a.Y2 || a.Z == a.Y2b))))
    return cudaErrorInvalidValue;  // a k-sum reads every k of its inputs
  const bool three = a.X2 != nullptr || (a.kmode != 0 && a.nk > 1);
  const size_t smem = (size_t)(three ? 3 : 2) * L * sizeof(double2);
  cudaError_t e = cudaFuncSetAttribute(zcorrconv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const long long total = (long long)a.nk * a.nseries;
  const long long g = total < 65535LL * 16 ? total : 65535LL * 16;
  zcorrconv_kernel<<<(unsigned)g, FFT_NT, smem, s>>>(a, tw);
  count_launch();
  return cudaGetLastError();
}

namespace {
cudaError_t packed_launch(GwFusedArgs& a, int* smem) {
  if (a.nseries <= 0) return cudaSuccess;
  int L = 1, logL = 0;
  while (L < 2 * a.n) { L <<= 1; ++logL; }
  if (L > LMAX) return cudaErrorInvalidValue;
  a.L = L;
  a.logL = logL;
  *smem = 3 * L * (int)sizeof(double2);
  return cudaSuccess;
}
}  // namespace

cudaError_t gw_polarization_packed(GwFusedArgs a, const double2* tw, cudaStream_t s) {
  int smem = 0;
  cudaError_t e = packed_launch(a, &smem);
  if (e != cudaSuccess || a.nseries <= 0) return e;
  e = cudaFuncSetAttribute(gw_pol_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long long g = a.nseries < 65535LL * 16 ? a.nseries : 65535LL * 16;
  gw_pol_kernel<<<(unsigned)g, FFT_NT, smem, s>>>(a, tw);
  count_launch();
  return cudaGetLastError();
}

cudaError_t gw_selfenergy_packed(GwFusedArgs a, const double2* tw, cudaStream_t s) {
  int smem = 0;
  cudaError_t e = packed_launch(a, &smem);
  if (e != cudaSuccess || a.nseries <= 0) return e;
  e = cudaFuncSetAttribute(gw_sig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long long g = a.nseries < 65535LL * 16 ? a.nseries : 65535LL * 16;
  gw_sig_kernel<<<(unsigned)g, FFT_NT, smem, s>>>(a, tw);
  count_launch();
  return cudaGetLastError();
}

cudaError_t gw_sigma_post(int nm, long long nblocks, double2* SR, double2* SL, double2* SG,
                          cudaStream_t s) {
  const long long g = nblocks < 65535LL * 8 ? nblocks : 65535LL * 8;
  sigma_post_kernel<<<(unsigned)g, 256, 0, s>>>(nm, nblocks, SR, SL, SG);
  count_launch();
  return cudaGetLastError();
}

cudaError_t gw_band_zero(int nm, long long nblocks, int ndiag, double2* A, cudaStream_t s,
                         long long bstride) {
  if (ndiag < 0 || nblocks <= 0) return cudaSuccess;
  const long long nm2 = nm * (long long)nm, count = nblocks * nm2;
  band_zero_kernel<<<g1(count), 256, 0, s>>>(nm, count, bstride ? bstride : nm2, ndiag, A);
  count_launch();
  return cudaGetLastError();
}

cudaError_t gw_residual(long long count, const double2* nl, const double2* ol, const double2* ng,
                        const double2* og, double* sums, cudaStream_t s) {
  residual_kernel<<<g1(count) > 1024 ? 1024 : g1(count), 256, 0, s>>>(count, nl, ol, ng, og, sums);
  count_launch();
  return cudaGetLastError();
}

cudaError_t photon_shift_sum(long long per, long long nE, int nop, int halo, double scale,
                             const double2* G, double2* A, cudaStream_t s) {
  photon_shift_sum_kernel<<<g1(nE * per), 256, 0, s>>>(per, nE, nop, halo, scale, G, A);
  count_launch();
  return cudaGetLastError();
}

cudaError_t photon_retarded(long long count, const double2* SL, const double2* SG, double2* SR,
                            cudaStream_t s) {
  photon_retarded_kernel<<<g1(count), 256, 0, s>>>(count, SL, SG, SR);
  count_launch();
  return cudaGetLastError();
}

cudaError_t gw_mix(long long count, double alpha, double2* S, const double2* N, cudaStream_t s) {
  mix_kernel<<<g1(count), 256, 0, s>>>(count, alpha, S, N);
  count_launch();
  return cudaGetLastError();
}

}  // namespace qt
