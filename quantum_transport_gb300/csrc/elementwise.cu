// O(n^2) per-block helpers of the RGF sweep: the zaxpy/zscal/zcopy chains,
// the contact broadening -(Sigma - Sigma^+) f (src/cuda_rgf_mod.f90:113,242,
// 254-264, 387-396), the Sancho error measure (src/cuda_rgf_mod.f90:721-726)
// and the diagonal traces behind tr/tre (src/cuda_rgf_mod.f90:271-277,
// 403-407) and the per-cell LDOS/n/p spectra (src/output_mod.f90:37-59).
//
// Every helper is templated on the block storage: double2 (complex128,
// arithmetic on the FP64 pipes) or float2 (complex64, FP32 arithmetic -- the
// split-precision sweep, where GB300's slow FP64 pipes must stay idle).
// Reductions (traces, sums) always accumulate in double.
#include "qt_common.cuh"
#include "qt_kernels.h"

namespace qt {

namespace {

constexpr int NT = 256;

template <typename TC> struct CT;
template <> struct CT<double2> {
  using R = double;
};
template <> struct CT<float2> {
  using R = float;
};

template <typename TC> __device__ __forceinline__ TC mk(double a, double b);
template <> __device__ __forceinline__ double2 mk<double2>(double a, double b) {
  return make_double2(a, b);
}
template <> __device__ __forceinline__ float2 mk<float2>(double a, double b) {
  return make_float2((float)a, (float)b);
}
template <typename TC> __device__ __forceinline__ TC tadd(TC a, TC b) {
  TC r; r.x = a.x + b.x; r.y = a.y + b.y; return r;
}
template <typename TC> __device__ __forceinline__ TC tsub(TC a, TC b) {
  TC r; r.x = a.x - b.x; r.y = a.y - b.y; return r;
}
template <typename TC, typename R> __device__ __forceinline__ TC tmul(R ar, R ai, TC b) {
  TC r; r.x = ar * b.x - ai * b.y; r.y = ar * b.y + ai * b.x; return r;
}
template <typename TC> __device__ __forceinline__ TC tconj(TC a) { a.y = -a.y; return a; }

inline unsigned grid_for(long long batch) {
  return (unsigned)(batch < 65535LL * 8 ? batch : 65535LL * 8);
}

template <typename TC>
__global__ void zaxpby_kernel(int n, long long batch, BatchRef X, double ar, double ai, BatchRef W,
                              double br, double bi, BatchRef Z, BatchRef Y,
                              const unsigned char* active) {
  using R = typename CT<TC>::R;
  // coefficients +-1 (every use in the sweeps): sign flips instead of complex products,
  // which on GB300's FP64 pipes are the cost of this kernel
  const int sa = (ai == 0.0 && (ar == 1.0 || ar == -1.0)) ? (ar > 0 ? 1 : -1) : 0;
  const int sb = (bi == 0.0 && (br == 1.0 || br == -1.0)) ? (br > 0 ? 1 : -1) : 0;
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    if (active && !active[b]) continue;
    const TC* x = X.p ? batch_ptr<const TC>(X, b) : nullptr;
    const TC* w = W.p ? batch_ptr<const TC>(W, b) : nullptr;
    TC* y = batch_ptr<TC>(Y, b);
    TC z = mk<TC>(0.0, 0.0);
    if (Z.p) {
      const double2 zz = *batch_ptr<const double2>(Z, b);  // shifts are always complex128
      z = mk<TC>(zz.x, zz.y);
    }
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      TC v = mk<TC>(0.0, 0.0);
      if (x) {
        const TC a = x[i + (long long)j * X.ld];
        v = sa > 0 ? a : sa < 0 ? mk<TC>(-(double)a.x, -(double)a.y) : tmul<TC, R>((R)ar, (R)ai, a);
      }
      if (w) {
        const TC c = w[i + (long long)j * W.ld];
        v = tadd(v, sb > 0 ? c : sb < 0 ? mk<TC>(-(double)c.x, -(double)c.y)
                                        : tmul<TC, R>((R)br, (R)bi, c));
      }
      if (i == j) v = tadd(v, z);
      y[i + (long long)j * Y.ld] = v;
    }
  }
}

template <typename TC>
__global__ void zantiherm_kernel(int n, long long batch, BatchRef X, double cr, double ci,
                                 BatchRef W, BatchRef Y) {
  using R = typename CT<TC>::R;
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* x = batch_ptr<const TC>(X, b);
    const TC* w = W.p ? batch_ptr<const TC>(W, b) : nullptr;
    TC* y = batch_ptr<TC>(Y, b);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const TC d = tsub(x[i + (long long)j * X.ld], tconj(x[j + (long long)i * X.ld]));
      TC v = tmul<TC, R>((R)cr, (R)ci, d);
      if (w) v = tadd(v, w[i + (long long)j * W.ld]);
      y[i + (long long)j * Y.ld] = v;
    }
  }
}

template <typename TC>
__global__ void zdagger_kernel(int n, long long batch, BatchRef X, BatchRef Y) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* x = batch_ptr<const TC>(X, b);
    TC* y = batch_ptr<TC>(Y, b);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      y[i + (long long)j * Y.ld] = tconj(x[j + (long long)i * X.ld]);
    }
  }
}

__device__ double block_sum(double v) {
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;  // valid in thread 0
}

// Y1_b += X_b and Y2_b += X_b in one pass over X (the decimation's paired updates)
template <typename TC>
__global__ void zadd2_kernel(int n, long long batch, BatchRef X, BatchRef Y1, BatchRef Y2,
                             const unsigned char* active) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    if (active && !active[b]) continue;
    const TC* x = batch_ptr<const TC>(X, b);
    TC* y1 = batch_ptr<TC>(Y1, b);
    TC* y2 = batch_ptr<TC>(Y2, b);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const TC v = x[i + (long long)j * X.ld];
      TC* p1 = y1 + i + (long long)j * Y1.ld;
      TC* p2 = y2 + i + (long long)j * Y2.ld;
      *p1 = tadd(*p1, v);
      *p2 = tadd(*p2, v);
    }
  }
}

// sum_ij |X_ij| per block, compared against `near` by its user.  The moduli come from FP32
// square roots of the components scaled by 2^40: relative error <= 3 2^-24 where the
// squares stay normal (moduli above 1e-31), absolute error below 1e-31 under that, inf
// above 3e26.  GB300's FP64 square root is the slow part of an FP64 sum.  Where these
// bounds leave the comparison with `near` undecided, the sum is redone with FP64 square
// roots, so every comparison with `near` comes out as with the FP64 sum.
template <typename TC>
__global__ void zabssum_kernel(int n, long long batch, BatchRef X, double* out,
                               const unsigned char* active, double near) {
  __shared__ int redo;
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    if (active && !active[b]) continue;
    const TC* x = batch_ptr<const TC>(X, b);
    double s = 0.0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const TC v = x[e % n + (long long)(e / n) * X.ld];
      const float fr = (float)v.x * 0x1p40f, fi = (float)v.y * 0x1p40f;
      s += (double)sqrtf(fmaf(fr, fr, fi * fi)) * 0x1p-40;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) {
      const double slack = (double)n * n * 1e-31;
      redo = !(s * (1.0 + 5e-7) + slack < near || s * (1.0 - 5e-7) - slack > near);
    }
    __syncthreads();
    if (redo) {
      double t = 0.0;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const TC v = x[e % n + (long long)(e / n) * X.ld];
        t += sqrt((double)v.x * v.x + (double)v.y * v.y);
      }
      s = block_sum(t);
    }
    if (threadIdx.x == 0) out[b] = s;
    __syncthreads();  // `redo` is rewritten for the next block
  }
}

// out_b = sign * Re( f Tr[K Y1] - (f-1) Tr[K Y2] ),  K = -(X - X^+), f = fermi[b]
// (src/cuda_rgf_mod.f90:256-277 with Y1 = G^>, Y2 = G^<)
template <typename TC>
__global__ void ztrace_current_kernel(int n, long long batch, BatchRef X, BatchRef Y1,
                                      BatchRef Y2, double sign, const double* fermi, double* out) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* x = batch_ptr<const TC>(X, b);
    const TC* y1 = batch_ptr<const TC>(Y1, b);
    const TC* y2 = batch_ptr<const TC>(Y2, b);
    const double f = fermi[b];
    double s = 0.0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const TC xa = x[j + (long long)i * X.ld], xb = x[i + (long long)j * X.ld];
      const double kx = (double)xa.x - xb.x, ky = -(double)xa.y - xb.y;  // conj(X(j,i)) - X(i,j)
      const TC u = y1[j + (long long)i * Y1.ld], v = y2[j + (long long)i * Y2.ld];
      const double t1 = kx * u.x - ky * u.y, t2 = kx * v.x - ky * v.y;
      s += f * t1 - (f - 1.0) * t2;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) out[b] = sign * s;
  }
}

template <typename TC>
__global__ void ztrace_prod_kernel(int n, long long batch, BatchRef X, BatchRef Y, double scale,
                                   double* out) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* x = batch_ptr<const TC>(X, b);
    const TC* y = batch_ptr<const TC>(Y, b);
    double s = 0.0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const TC u = x[i + (long long)j * X.ld], v = y[j + (long long)i * Y.ld];
      s += (double)u.x * v.x - (double)u.y * v.y;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) out[b] = scale * s;
  }
}

// Bond current of one slab pair: T1 (nl x nq), H (nq x nl), A (nq x nl);
// out = scale * 2 (-Re sum_ij T1(i,j) H(j,i) + Re sum_ab conj(H(a,b)) A(a,b)),
// the first sum skipped when T1 is null.
template <typename TC>
__global__ void zbond_trace_kernel(int nl, int nq, long long batch, BatchRef T1, BatchRef H,
                                   BatchRef A, double scale, double* out, long long ostride,
                                   long long ooff) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* t1 = T1.p ? batch_ptr<const TC>(T1, b) : nullptr;
    const TC* h = batch_ptr<const TC>(H, b);
    const TC* a = batch_ptr<const TC>(A, b);
    double s = 0.0;
    for (int e = threadIdx.x; e < nl * nq; e += blockDim.x) {
      if (t1) {
        const int i = e % nl, j = e / nl;
        const TC u = t1[i + (long long)j * T1.ld], v = h[j + (long long)i * H.ld];
        s -= (double)u.x * v.x - (double)u.y * v.y;
      }
      const int r = e % nq, c = e / nq;
      const TC hv = h[r + (long long)c * H.ld], av = a[r + (long long)c * A.ld];
      s += (double)hv.x * av.x + (double)hv.y * av.y;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) out[b * ostride + ooff] = 2.0 * scale * s;
  }
}

template <typename TC>
__global__ void zdiag_kernel(int n, long long batch, BatchRef X, double* out, long long ostride,
                             long long ooff) {
  const long long total = batch * n;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / n;
    const int i = (int)(t % n);
    const TC v = batch_ptr<const TC>(X, b)[i + (long long)i * X.ld];
    reinterpret_cast<double2*>(out)[b * ostride + ooff + i] = make_double2(v.x, v.y);
  }
}

// diag of G^> = G^< + (G - G^+): Y(i,i) + 2i Im X(i,i)
template <typename TC>
__global__ void zdiag_greater_kernel(int n, long long batch, BatchRef X, BatchRef Y, double* out,
                                     long long ostride, long long ooff) {
  const long long total = batch * n;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / n;
    const int i = (int)(t % n);
    const TC g = batch_ptr<const TC>(X, b)[i + (long long)i * X.ld];
    const TC l = batch_ptr<const TC>(Y, b)[i + (long long)i * Y.ld];
    reinterpret_cast<double2*>(out)[b * ostride + ooff + i] =
        make_double2(l.x, (double)l.y + 2.0 * (double)g.y);
  }
}

template <typename TC>
__global__ void zscale_add_kernel(int n, long long batch, BatchRef X, const double* f, BatchRef W,
                                  BatchRef Y) {
  using R = typename CT<TC>::R;
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* x = batch_ptr<const TC>(X, b);
    const TC* w = W.p ? batch_ptr<const TC>(W, b) : nullptr;
    TC* y = batch_ptr<TC>(Y, b);
    const R fb = (R)f[b];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const TC xv = x[i + (long long)j * X.ld];
      TC v;
      v.x = fb * xv.x;
      v.y = fb * xv.y;
      if (w) v = tadd(v, w[i + (long long)j * W.ld]);
      y[i + (long long)j * Y.ld] = v;
    }
  }
}

template <typename TS, typename TD>
__global__ void zconvert_kernel(int n, long long batch, BatchRef X, BatchRef Y) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TS* x = batch_ptr<const TS>(X, b);
    TD* y = batch_ptr<TD>(Y, b);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const TS v = x[i + (long long)j * X.ld];
      y[i + (long long)j * Y.ld] = mk<TD>((double)v.x, (double)v.y);
    }
  }
}

template <typename TC>
__global__ void zcheck_finite_kernel(int n, long long batch, BatchRef X, int* status) {
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    const TC* x = batch_ptr<const TC>(X, b);
    int bad = 0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const TC v = x[e % n + (long long)(e / n) * X.ld];
      if (!isfinite((double)v.x) || !isfinite((double)v.y)) bad = 1;
    }
    bad = __syncthreads_or(bad);
    if (bad && threadIdx.x == 0) atomicOr(&status[b], PT_NONFINITE);
  }
}

inline unsigned gdiag(long long total) {
  const long long g = (total + NT - 1) / NT;
  return (unsigned)(g < 65535LL * 16 ? (g < 1 ? 1 : g) : 65535LL * 16);
}

}  // namespace

template <typename TC>
cudaError_t zaxpby(int n, long long batch, BatchRef X, double ar, double ai, BatchRef W, double br,
                   double bi, BatchRef Z, BatchRef Y, const unsigned char* active, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zaxpby_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, ar, ai, W, br, bi, Z, Y, active);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zantiherm(int n, long long batch, BatchRef X, double cr, double ci, BatchRef W,
                      BatchRef Y, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zantiherm_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, cr, ci, W, Y);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zdagger(int n, long long batch, BatchRef X, BatchRef Y, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zdagger_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, Y);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zadd2(int n, long long batch, BatchRef X, BatchRef Y1, BatchRef Y2,
                  const unsigned char* active, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zadd2_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, Y1, Y2, active);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zabssum(int n, long long batch, BatchRef X, double* out, const unsigned char* active,
                    double near, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zabssum_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, out, active, near);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t ztrace_current(int n, long long batch, BatchRef X, BatchRef Y1, BatchRef Y2,
                           double sign, const double* fermi, double* out, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  ztrace_current_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, Y1, Y2, sign, fermi, out);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t ztrace_prod(int n, long long batch, BatchRef X, BatchRef Y, double scale, double* out,
                        cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  ztrace_prod_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, Y, scale, out);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zbond_trace(int nl, int nq, long long batch, BatchRef T1, BatchRef H, BatchRef A,
                        double scale, double* out, long long ostride, long long ooff,
                        cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zbond_trace_kernel<TC><<<grid_for(batch), NT, 0, s>>>(nl, nq, batch, T1, H, A, scale, out,
                                                        ostride, ooff);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zscale_add(int n, long long batch, BatchRef X, const double* f, BatchRef W, BatchRef Y,
                       cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zscale_add_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, f, W, Y);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zdiag(int n, long long batch, BatchRef X, double* out, long long ostride,
                  long long ooff, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zdiag_kernel<TC><<<gdiag(batch * n), NT, 0, s>>>(n, batch, X, out, ostride, ooff);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zdiag_greater(int n, long long batch, BatchRef X, BatchRef Y, double* out,
                          long long ostride, long long ooff, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zdiag_greater_kernel<TC><<<gdiag(batch * n), NT, 0, s>>>(n, batch, X, Y, out, ostride, ooff);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zcopy(int n, long long batch, BatchRef X, BatchRef Y, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zconvert_kernel<TC, TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, Y);
  count_launch();
  return cudaGetLastError();
}
template <typename TS, typename TD>
cudaError_t zconvert(int n, long long batch, BatchRef X, BatchRef Y, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zconvert_kernel<TS, TD><<<grid_for(batch), NT, 0, s>>>(n, batch, X, Y);
  count_launch();
  return cudaGetLastError();
}
template <typename TC>
cudaError_t zcheck_finite(int n, long long batch, BatchRef X, int* status, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zcheck_finite_kernel<TC><<<grid_for(batch), NT, 0, s>>>(n, batch, X, status);
  count_launch();
  return cudaGetLastError();
}

#define QT_INST(TC)                                                                               \
  template cudaError_t zaxpby<TC>(int, long long, BatchRef, double, double, BatchRef, double,     \
                                  double, BatchRef, BatchRef, const unsigned char*, cudaStream_t); \
  template cudaError_t zantiherm<TC>(int, long long, BatchRef, double, double, BatchRef,          \
                                     BatchRef, cudaStream_t);                                     \
  template cudaError_t zdagger<TC>(int, long long, BatchRef, BatchRef, cudaStream_t);             \
  template cudaError_t zadd2<TC>(int, long long, BatchRef, BatchRef, BatchRef,                   \
                                 const unsigned char*, cudaStream_t);                             \
  template cudaError_t zabssum<TC>(int, long long, BatchRef, double*, const unsigned char*,       \
                                   double, cudaStream_t);                                         \
  template cudaError_t ztrace_current<TC>(int, long long, BatchRef, BatchRef, BatchRef, double,   \
                                          const double*, double*, cudaStream_t);                  \
  template cudaError_t ztrace_prod<TC>(int, long long, BatchRef, BatchRef, double, double*,       \
                                       cudaStream_t);                                             \
  template cudaError_t zbond_trace<TC>(int, int, long long, BatchRef, BatchRef, BatchRef, double, \
                                      double*, long long, long long, cudaStream_t);              \
  template cudaError_t zscale_add<TC>(int, long long, BatchRef, const double*, BatchRef,          \
                                      BatchRef, cudaStream_t);                                    \
  template cudaError_t zdiag<TC>(int, long long, BatchRef, double*, long long, long long,         \
                                 cudaStream_t);                                                   \
  template cudaError_t zdiag_greater<TC>(int, long long, BatchRef, BatchRef, double*, long long,  \
                                         long long, cudaStream_t);                                \
  template cudaError_t zcopy<TC>(int, long long, BatchRef, BatchRef, cudaStream_t);               \
  template cudaError_t zcheck_finite<TC>(int, long long, BatchRef, int*, cudaStream_t);
QT_INST(double2)
QT_INST(float2)
template cudaError_t zconvert<double2, float2>(int, long long, BatchRef, BatchRef, cudaStream_t);
template cudaError_t zconvert<float2, double2>(int, long long, BatchRef, BatchRef, cudaStream_t);

}  // namespace qt
