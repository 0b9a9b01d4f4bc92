// Kernels of the SCBA mixing steps: the learned per-orbital step and its
// Pulay (DIIS) fallback.  The reference mixes linearly,
// Sigma <- Sigma + alpha (Sigma_new - Sigma) (src/gw_mod.f90:747-749); these
// kernels serve the mixing that replaces it.
//
// Layout: every self-energy is [nE][nx][nm*nm] complex128, column-major
// blocks (the layout of qt_gw_step).  An orbital o = l*nm + i is row/column i
// of slab l; its diagonal series is Im Sigma[e][l][i + i*nm] over e.
//
//  * mix_diag:     Im of the diagonal series of X^< and X^> -> [2][nE][norb]
//  * mix_features: per orbital, 64 Chebyshev coefficients of each of the
//                  last nhist residual series (< and >), scaled by the norm of
//                  the newest pair and clamped to +-8, plus the global residual
//                  and the orbital's residual decay: the network's input row
//  * mix_apply:    S + a_ij R + b_ij (S - S_prev) with a_ij = (a_i + a_j)/2,
//                  b_ij = (b_i + b_j)/2 from the per-orbital network outputs
//  * mix_gram / mix_combine: Pulay's residual Gram matrix and the affine
//                  combination of the history
#include <math.h>

#include "qt_abi.h"
#include "qt_kernels.h"

namespace qt {
namespace {

constexpr int NCOEF = 64;
constexpr int MAXVEC = 8;

struct PtrList {
  const double2* p[MAXVEC];
};

__global__ void mix_diag_kernel(int nE, int nx, int nm, const double2* XL, const double2* XG,
                                double* out) {
  const long long norb = (long long)nx * nm, nm2 = (long long)nm * nm;
  const long long total = 2 * (long long)nE * norb;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long q = t / ((long long)nE * norb), r = t % ((long long)nE * norb);
    const long long e = r / norb, o = r % norb;
    const long long l = o / nm, i = o % nm;
    const double2* X = q ? XG : XL;
    out[t] = X[(e * nx + l) * nm2 + i + i * nm].y;
  }
}

// one CTA per orbital; thread (s, m): series s = h*2 + q, coefficient m
__global__ void mix_features_kernel(int nE, long long norb, int nhist, const double* ring,
                                    const double* Qt, double log_residual, float* feats,
                                    int n_in) {
  extern __shared__ double red[];  // [nhist*2][NCOEF]
  const int t = threadIdx.x, s = t / NCOEF, m = t % NCOEF;
  for (long long o = blockIdx.x; o < norb; o += gridDim.x) {
    double c = 0.0;
    if (s < 2 * nhist) {
      const double* x = ring + (long long)s * nE * norb + o;
      for (int e = 0; e < nE; ++e) c += Qt[(long long)e * NCOEF + m] * x[(long long)e * norb];
      red[t] = c;
    }
    __syncthreads();
    // norms of the newest (h = 0) and previous (h = 1) residual pairs
    if (t == 0) {
      double n0 = 0.0, n1 = 0.0;
      for (int k = 0; k < 2 * NCOEF; ++k) n0 += red[k] * red[k];
      if (nhist > 1)
        for (int k = 2 * NCOEF; k < 4 * NCOEF; ++k) n1 += red[k] * red[k];
      red[2 * nhist * NCOEF] = sqrt(n0);
      red[2 * nhist * NCOEF + 1] = sqrt(n1);
    }
    __syncthreads();
    const double n0 = red[2 * nhist * NCOEF], n1 = red[2 * nhist * NCOEF + 1];
    float* f = feats + o * n_in;
    // an orbital whose newest residual vanishes would blow its older ones up: clamp to +-8
    if (s < 2 * nhist) f[t] = (float)fmax(-8.0, fmin(8.0, c / (n0 + 1e-300)));
    if (t == 0) {
      f[2 * nhist * NCOEF] = (float)(log_residual / 8.0);
      const double decay = (nhist > 1 && n1 > 0.0 && n0 > 0.0) ? log10(n0 / n1) : 0.0;
      f[2 * nhist * NCOEF + 1] = (float)fmax(-4.0, fmin(4.0, decay));
    }
    __syncthreads();
  }
}

__global__ void mix_apply_kernel(int nE, int nx, int nm, const float* ab, int ncols, float amax,
                                 float bmin, float bmax, const double2* S, const double2* R,
                                 const double2* Sp, double2* out) {
  const long long nm2 = (long long)nm * nm, total = (long long)nE * nx * nm2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long blk = t / nm2, w = t % nm2;
    const int l = (int)(blk % nx), i = (int)(w % nm), j = (int)(w / nm);
    const long long oi = (long long)l * nm + i, oj = (long long)l * nm + j;
    const float ai = fminf(fmaxf(ab[ncols * oi], 0.0f), amax);
    const float aj = fminf(fmaxf(ab[ncols * oj], 0.0f), amax);
    const float bi = ncols > 1 ? fminf(fmaxf(ab[ncols * oi + 1], bmin), bmax) : 0.0f;
    const float bj = ncols > 1 ? fminf(fmaxf(ab[ncols * oj + 1], bmin), bmax) : 0.0f;
    const double a = 0.5 * ((double)ai + aj), b = 0.5 * ((double)bi + bj);
    const double2 s = S[t], r = R[t], p = Sp ? Sp[t] : s;
    out[t] = make_double2(s.x + a * r.x + b * (s.x - p.x), s.y + a * r.y + b * (s.y - p.y));
  }
}

// G[i][j] += sum Re(conj(X_i) X_j) over both lists (lower triangle, i >= j)
__global__ void mix_gram_kernel(long long count, int k, PtrList L, PtrList G2, double* G) {
  double acc[MAXVEC * (MAXVEC + 1) / 2];
#pragma unroll
  for (int q = 0; q < MAXVEC * (MAXVEC + 1) / 2; ++q) acc[q] = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    double2 a[MAXVEC], b[MAXVEC];
#pragma unroll
    for (int i = 0; i < MAXVEC; ++i) {
      if (i < k) {
        a[i] = L.p[i][t];
        b[i] = G2.p[i][t];
      }
    }
    int q = 0;
#pragma unroll
    for (int i = 0; i < MAXVEC; ++i)
#pragma unroll
      for (int j = 0; j <= i; ++j, ++q)
        if (i < k) acc[q] += a[i].x * a[j].x + a[i].y * a[j].y + b[i].x * b[j].x + b[i].y * b[j].y;
  }
  int q = 0;
#pragma unroll
  for (int i = 0; i < MAXVEC; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j, ++q) {
      if (i >= k) continue;
      double v = acc[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if ((threadIdx.x & 31) == 0) atomicAdd(&G[i * k + j], v);
    }
}

struct CoefList {
  double c[MAXVEC];
};

// out = sum_i c_i (X_i + alpha R_i)
__global__ void mix_combine_kernel(long long count, int k, CoefList c, PtrList X, PtrList R,
                                   double alpha, double2* out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
#pragma unroll
    for (int i = 0; i < MAXVEC; ++i) {
      if (i < k) {
        const double2 x = X.p[i][t], r = R.p[i][t];
        s.x += c.c[i] * (x.x + alpha * r.x);
        s.y += c.c[i] * (x.y + alpha * r.y);
      }
    }
    out[t] = s;
  }
}

inline unsigned grid_of(long long n, long long cap = 8192) {
  long long g = (n + 255) / 256;
  return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

qt_status launched(cudaStream_t s, unsigned flags) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(s));
  return QT_OK;
}

}  // namespace
}  // namespace qt

extern "C" qt_status qt_mix_diag(qt_ctx* ctx, int nE, int nx, int nm, const double* XL,
                                 const double* XG, double* out, unsigned flags) {
  if (!ctx || !XL || !XG || !out || nE <= 0 || nx <= 0 || nm <= 0)
    QT_FAIL(QT_ERR_ARG, "bad mix_diag arguments");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t s = qt::ctx_stream(ctx);
  const long long total = 2LL * nE * nx * nm;
  qt::mix_diag_kernel<<<qt::grid_of(total), 256, 0, s>>>(
      nE, nx, nm, reinterpret_cast<const double2*>(XL), reinterpret_cast<const double2*>(XG), out);
  return qt::launched(s, flags);
}

extern "C" qt_status qt_mix_features(qt_ctx* ctx, int nE, int64_t norb, int nhist,
                                     const double* ring, const double* Qt, double log_residual,
                                     float* feats, unsigned flags) {
  if (!ctx || !ring || !Qt || !feats || nE <= 0 || norb <= 0 || nhist < 1 || nhist > 3)
    QT_FAIL(QT_ERR_ARG, "bad mix_features arguments (1 <= nhist <= 3)");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t s = qt::ctx_stream(ctx);
  const int threads = 2 * nhist * qt::NCOEF;
  const size_t smem = (size_t)(threads + 2) * sizeof(double);
  const unsigned grid = (unsigned)(norb < 65535 * 4 ? norb : 65535 * 4);
  qt::mix_features_kernel<<<grid, threads, smem, s>>>(nE, norb, nhist, ring, Qt, log_residual,
                                                      feats, 2 * nhist * qt::NCOEF + 2);
  return qt::launched(s, flags);
}

extern "C" qt_status qt_mix_apply(qt_ctx* ctx, int nE, int nx, int nm, const float* ab,
                                  int ncols, double alpha_max, double beta_min, double beta_max,
                                  const double* S, const double* R, const double* S_prev,
                                  double* out, unsigned flags) {
  if (!ctx || !ab || !S || !R || !out || nE <= 0 || nx <= 0 || nm <= 0 || ncols < 1 ||
      ncols > 2)
    QT_FAIL(QT_ERR_ARG, "bad mix_apply arguments");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t s = qt::ctx_stream(ctx);
  const long long total = (long long)nE * nx * nm * nm;
  qt::mix_apply_kernel<<<qt::grid_of(total), 256, 0, s>>>(
      nE, nx, nm, ab, ncols, (float)alpha_max, (float)beta_min, (float)beta_max,
      reinterpret_cast<const double2*>(S), reinterpret_cast<const double2*>(R),
      reinterpret_cast<const double2*>(S_prev), reinterpret_cast<double2*>(out));
  return qt::launched(s, flags);
}

extern "C" qt_status qt_mix_gram(qt_ctx* ctx, int64_t count, int k, const double* const* XL,
                                 const double* const* XG, double* G_host) {
  if (!ctx || !XL || !XG || !G_host || count <= 0 || k < 1 || k > qt::MAXVEC)
    QT_FAIL(QT_ERR_ARG, "bad mix_gram arguments (1 <= k <= 8)");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t s = qt::ctx_stream(ctx);
  qt::PtrList a{}, b{};
  for (int i = 0; i < k; ++i) {
    if (!XL[i] || !XG[i]) QT_FAIL(QT_ERR_ARG, "null vector");
    a.p[i] = reinterpret_cast<const double2*>(XL[i]);
    b.p[i] = reinterpret_cast<const double2*>(XG[i]);
  }
  double* G = nullptr;
  QT_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&G), sizeof(double) * k * k, s));
  cudaMemsetAsync(G, 0, sizeof(double) * k * k, s);
  qt::mix_gram_kernel<<<qt::grid_of(count, 1024), 256, 0, s>>>(count, k, a, b, G);
  qt::count_launch();
  cudaMemcpyAsync(G_host, G, sizeof(double) * k * k, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(G, s);
  QT_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < k; ++i)
    for (int j = i + 1; j < k; ++j) G_host[i * k + j] = G_host[j * k + i];
  return QT_OK;
}

extern "C" qt_status qt_mix_combine(qt_ctx* ctx, int64_t count, int k, const double* coef,
                                    const double* const* X, const double* const* R, double alpha,
                                    double* out, unsigned flags) {
  if (!ctx || !coef || !X || !R || !out || count <= 0 || k < 1 || k > qt::MAXVEC)
    QT_FAIL(QT_ERR_ARG, "bad mix_combine arguments (1 <= k <= 8)");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t s = qt::ctx_stream(ctx);
  qt::PtrList x{}, r{};
  qt::CoefList c{};
  for (int i = 0; i < k; ++i) {
    if (!X[i] || !R[i]) QT_FAIL(QT_ERR_ARG, "null vector");
    x.p[i] = reinterpret_cast<const double2*>(X[i]);
    r.p[i] = reinterpret_cast<const double2*>(R[i]);
    c.c[i] = coef[i];
  }
  qt::mix_combine_kernel<<<qt::grid_of(count), 256, 0, s>>>(count, k, c, x, r, alpha,
                                                            reinterpret_cast<double2*>(out));
  return qt::launched(s, flags);
}
