// Batched complex block inversion by Gauss-Jordan elimination with partial
// (row) pivoting, one CTA per block.
//
// Replaces the reference's LU inverse ``invert`` -- zgetrf + zgetrs against
// the identity (src/cuda_rgf_mod.f90:624-654, :118-125, :159-164;
// src/linalg.f90:42-62 with zgetri).  Pivot choice follows LAPACK's izamax
// measure |re| + |im| with the first maximal row winning.  Unlike the
// reference (abort() at src/cuda_rgf_mod.f90:180-187, or zeroing A at
// src/linalg.f90:50-58) a zero or non-finite pivot only raises PT_SINGULAR in
// the per-point status; the batch continues.
//
//  * zinv_f64: FP64 arithmetic, block in global memory (L2 resident).  FP64
//    throughput bounds it on GB300; it is the plain-FP64 path.
//  * zinv_f32: the block is converted to complex64 and eliminated entirely in
//    shared memory (n <= 128: 128 KB), the result is written back as FP64.
//    The split-precision path refines it with one residual step
//    X <- X + X (I - A X) computed by the tensor-core GEMM.
#include "qt_common.cuh"
#include "qt_kernels.h"

namespace qt {

namespace {

constexpr int NT64 = 256;

__device__ __forceinline__ double cabs1(cd v) { return fabs(v.x) + fabs(v.y); }
__device__ __forceinline__ cd crecip(cd p) {
  const double d = p.x * p.x + p.y * p.y;
  return cd{p.x / d, -p.y / d};
}

template <int NT>
__device__ __forceinline__ void block_argmax(double& v, int& idx, double* rv, int* ri) {
  // warp reduce, then across warps; ties -> smaller index
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, v, o);
    const int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  if (lane == 0) { rv[w] = v; ri[w] = idx; }
  __syncthreads();
  if (w == 0) {
    v = lane < NT / 32 ? rv[lane] : -1.0;
    idx = lane < NT / 32 ? ri[lane] : 0x7fffffff;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_down_sync(0xffffffffu, v, o);
      const int oi = __shfl_down_sync(0xffffffffu, idx, o);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    if (lane == 0) { rv[0] = v; ri[0] = idx; }
  }
  __syncthreads();
  v = rv[0];
  idx = ri[0];
  __syncthreads();
}

__global__ __launch_bounds__(NT64) void zinv_f64_kernel(InvArgs a) {
  extern __shared__ double2 smem_raw[];
  const int n = a.n;
  cd* colk = reinterpret_cast<cd*>(smem_raw);
  cd* rowk = colk + n;
  int* perm = reinterpret_cast<int*>(rowk + n);
  __shared__ double rv[32];
  __shared__ int ri[32];
  const int tid = threadIdx.x;
  for (long long b = blockIdx.x; b < a.batch; b += gridDim.x) {
    if (a.active && !a.active[b]) continue;
    const cd* A = batch_ptr<const cd>(a.A, b);
    cd* X = batch_ptr<cd>(a.X, b);
    const int lda = a.A.ld, ld = a.X.ld;
    if ((const void*)A != (const void*)X || lda != ld) {
      for (int e = tid; e < n * n; e += NT64) X[e % n + (long long)(e / n) * ld] = A[e % n + (long long)(e / n) * lda];
      __syncthreads();
    }
    bool bad = false;
    for (int k = 0; k < n; ++k) {
      double best = -1.0;
      int bi = 0x7fffffff;
      for (int i = k + tid; i < n; i += NT64) {
        const double m = cabs1(X[i + (long long)k * ld]);
        if (m > best || (m == best && i < bi)) { best = m; bi = i; }
      }
      block_argmax<NT64>(best, bi, rv, ri);
      if (!(best > 0.0) || !isfinite(best)) { bad = true; bi = k; }
      const int p = bi;
      if (tid == 0) perm[k] = p;
      if (p != k) {
        for (int j = tid; j < n; j += NT64) {
          const cd t = X[k + (long long)j * ld];
          X[k + (long long)j * ld] = X[p + (long long)j * ld];
          X[p + (long long)j * ld] = t;
        }
      }
      __syncthreads();
      const cd piv = X[k + (long long)k * ld];
      const cd inv = (piv.x == 0.0 && piv.y == 0.0) ? cd{0.0, 0.0} : crecip(piv);
      for (int i = tid; i < n; i += NT64) colk[i] = X[i + (long long)k * ld];
      for (int j = tid; j < n; j += NT64) rowk[j] = (j == k) ? inv : cmul(X[k + (long long)j * ld], inv);
      __syncthreads();
      for (int e = tid; e < n * n; e += NT64) {
        const int i = e % n, j = e / n;
        cd* x = &X[i + (long long)j * ld];
        if (i == k) *x = rowk[j];
        else if (j == k) *x = cmul(cd{-colk[i].x, -colk[i].y}, inv);
        else {
          cd v = *x;
          const cd c = colk[i], r = rowk[j];
          v.x = fma(-c.x, r.x, v.x); v.x = fma(c.y, r.y, v.x);
          v.y = fma(-c.x, r.y, v.y); v.y = fma(-c.y, r.x, v.y);
          *x = v;
        }
      }
      __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k) {
        for (int i = tid; i < n; i += NT64) {
          const cd t = X[i + (long long)k * ld];
          X[i + (long long)k * ld] = X[i + (long long)p * ld];
          X[i + (long long)p * ld] = t;
        }
      }
      __syncthreads();
    }
    if (bad && tid == 0 && a.status) atomicOr(&a.status[b], PT_SINGULAR);
    __syncthreads();
  }
}

// ---------------------------------------------------------------- FP32
constexpr int NT32 = 512;

__device__ __forceinline__ float2 to_f2(double2 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ float2 to_f2(float2 v) { return v; }
template <typename TC> __device__ __forceinline__ TC from_f2(float2 v);
template <> __device__ __forceinline__ double2 from_f2<double2>(float2 v) {
  return make_double2(v.x, v.y);
}
template <> __device__ __forceinline__ float2 from_f2<float2>(float2 v) { return v; }

template <typename TC>
__global__ __launch_bounds__(NT32) void zinv_f32_kernel(InvArgs a) {
  extern __shared__ float2 sm32[];
  const int n = a.n;
  float2* M = sm32;               // n*n, column-major, ld = n
  float2* colk = M + n * n;       // n
  float2* rowk = colk + n;        // n
  int* perm = reinterpret_cast<int*>(rowk + n);
  __shared__ double rv[32];
  __shared__ int ri[32];
  const int tid = threadIdx.x;
  for (long long b = blockIdx.x; b < a.batch; b += gridDim.x) {
    if (a.active && !a.active[b]) continue;
    const TC* A = batch_ptr<const TC>(a.A, b);
    TC* X = batch_ptr<TC>(a.X, b);
    const int lda = a.A.ld, ld = a.X.ld;
    for (int e = tid; e < n * n; e += NT32) M[e] = to_f2(A[e % n + (long long)(e / n) * lda]);
    __syncthreads();
    bool bad = false;
    for (int k = 0; k < n; ++k) {
      double best = -1.0;
      int bi = 0x7fffffff;
      for (int i = k + tid; i < n; i += NT32) {
        const float2 v = M[i + k * n];
        const double m = (double)(fabsf(v.x) + fabsf(v.y));
        if (m > best || (m == best && i < bi)) { best = m; bi = i; }
      }
      block_argmax<NT32>(best, bi, rv, ri);
      if (!(best > 0.0) || !isfinite(best)) { bad = true; bi = k; }
      const int p = bi;
      if (tid == 0) perm[k] = p;
      if (p != k) {
        for (int j = tid; j < n; j += NT32) {
          const float2 t = M[k + j * n];
          M[k + j * n] = M[p + j * n];
          M[p + j * n] = t;
        }
      }
      __syncthreads();
      const float2 piv = M[k + k * n];
      const float d = piv.x * piv.x + piv.y * piv.y;
      const float2 inv = d == 0.f ? make_float2(0.f, 0.f) : make_float2(piv.x / d, -piv.y / d);
      for (int i = tid; i < n; i += NT32) colk[i] = M[i + k * n];
      for (int j = tid; j < n; j += NT32) {
        const float2 r = M[k + j * n];
        rowk[j] = (j == k) ? inv : make_float2(r.x * inv.x - r.y * inv.y, r.x * inv.y + r.y * inv.x);
      }
      __syncthreads();
      for (int e = tid; e < n * n; e += NT32) {
        const int i = e % n, j = e / n;
        float2 v = M[e];
        const float2 c = colk[i], r = rowk[j];
        if (i == k) v = r;
        else if (j == k) v = make_float2(-(c.x * inv.x - c.y * inv.y), -(c.x * inv.y + c.y * inv.x));
        else {
          v.x = fmaf(-c.x, r.x, v.x); v.x = fmaf(c.y, r.y, v.x);
          v.y = fmaf(-c.x, r.y, v.y); v.y = fmaf(-c.y, r.x, v.y);
        }
        M[e] = v;
      }
      __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k) {
        for (int i = tid; i < n; i += NT32) {
          const float2 t = M[i + k * n];
          M[i + k * n] = M[i + p * n];
          M[i + p * n] = t;
        }
      }
      __syncthreads();
    }
    for (int e = tid; e < n * n; e += NT32) {
      const float2 v = M[e];
      X[e % n + (long long)(e / n) * ld] = from_f2<TC>(v);
    }
    if (bad && tid == 0 && a.status) atomicOr(&a.status[b], PT_SINGULAR);
    __syncthreads();
  }
}

long long grid_for(long long batch) { return batch < 65535 * 4 ? batch : 65535 * 4; }

}  // namespace

cudaError_t zinv_f64(const InvArgs& a, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  const size_t sm = (size_t)a.n * 2 * sizeof(cd) + (size_t)a.n * sizeof(int);
  zinv_f64_kernel<<<(unsigned)grid_for(a.batch), NT64, sm, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

template <typename TC>
cudaError_t zinv_f32(const InvArgs& a, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (a.n > 128) return cudaErrorInvalidValue;
  const size_t sm = (size_t)a.n * a.n * sizeof(float2) + (size_t)a.n * 2 * sizeof(float2) +
                    (size_t)a.n * sizeof(int);
  cudaError_t e = cudaFuncSetAttribute(zinv_f32_kernel<TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sm);
  if (e != cudaSuccess) return e;
  zinv_f32_kernel<TC><<<(unsigned)grid_for(a.batch), NT32, sm, s>>>(a);
  count_launch();
  return cudaGetLastError();
}
template cudaError_t zinv_f32<double2>(const InvArgs&, cudaStream_t);
template cudaError_t zinv_f32<float2>(const InvArgs&, cudaStream_t);

}  // namespace qt
