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

__device__ __forceinline__ cd to_cd(double2 v) { return cd{v.x, v.y}; }
__device__ __forceinline__ cd to_cd(float2 v) { return cd{v.x, v.y}; }

// FP64 Gauss-Jordan.  TC = double2: in place in X.  TC = float2 (complex64 storage): the
// block is eliminated in the complex128 workspace W (entry b at W + b * wst, ld n) and
// written back to X as complex64.
template <typename TC>
__global__ __launch_bounds__(NT64) void zinv_f64_kernel(InvArgs a, cd* W, long long wst) {
  extern __shared__ double2 smem_raw[];
  const int n = a.n;
  cd* colk = reinterpret_cast<cd*>(smem_raw);
  cd* rowk = colk + n;
  int* perm = reinterpret_cast<int*>(rowk + n);
  __shared__ double rv[32];
  __shared__ int ri[32];
  const int tid = threadIdx.x;
  constexpr bool wide = sizeof(TC) == 16;
  for (long long b = blockIdx.x; b < a.batch; b += gridDim.x) {
    if (a.active && !a.active[b]) continue;
    const TC* A = batch_ptr<const TC>(a.A, b);
    TC* Xs = batch_ptr<TC>(a.X, b);
    cd* X = wide ? reinterpret_cast<cd*>(Xs) : W + b * wst;
    const int lda = a.A.ld, ld = wide ? a.X.ld : n;
    if (!wide || (const void*)A != (const void*)X || lda != ld) {
      for (int e = tid; e < n * n; e += NT64)
        X[e % n + (long long)(e / n) * ld] = to_cd(A[e % n + (long long)(e / n) * lda]);
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
    if constexpr (!wide) {
      for (int e = tid; e < n * n; e += NT64) {
        const cd v = X[e % n + (long long)(e / n) * n];
        Xs[e % n + (long long)(e / n) * a.X.ld] = make_float2((float)v.x, (float)v.y);
      }
    }
    if (bad && tid == 0 && a.status) atomicOr(&a.status[b], PT_SINGULAR);
    __syncthreads();
  }
}

// flag[b] = active[b] && (||R_b||_F > tol or non-finite); *count += flagged entries
template <typename TC>
__global__ void zinv_guard_kernel(int n, long long batch, BatchRef R, const unsigned char* active,
                                  double tol, unsigned char* flag, int* count) {
  __shared__ double part[32];
  __shared__ bool undecided;
  for (long long b = blockIdx.x; b < batch; b += gridDim.x) {
    if (active && !active[b]) {
      if (threadIdx.x == 0) flag[b] = 0;
      continue;
    }
    const TC* r = batch_ptr<const TC>(R, b);
    // ||R||_F^2 against tol^2.  Complex64 residuals: FP32 squares summed in FP32 per thread
    // (relative error below 1e-4 for the <= 576 terms a thread adds at n <= 384; the FP64
    // pipes are the cost of the FP64 sum), the FP64 sum only where that leaves the
    // comparison undecided.  Complex128 residuals: the FP64 sum.
    bool exact = sizeof(TC) == 16;
    double t = 0.0;
    for (int pass = exact ? 1 : 0; pass < 2; ++pass) {
      double s = 0.0;
      if (pass == 0) {
        float f = 0.f;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
          const TC v = r[e % n + (long long)(e / n) * R.ld];
          f = fmaf((float)v.x, (float)v.x, fmaf((float)v.y, (float)v.y, f));
        }
        s = f;
      } else {
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
          const TC v = r[e % n + (long long)(e / n) * R.ld];
          s += (double)v.x * v.x + (double)v.y * v.y;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
      __syncthreads();
      if (threadIdx.x == 0) {
        t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        // squares of moduli below 1e-19 may be lost in FP32: 2e-38 each at most
        const double tt = tol * tol, slack = (double)n * n * 2e-38;
        undecided = pass == 0 && !(t * (1.0 + 1e-4) + slack <= tt || t * (1.0 - 1e-4) - slack > tt);
      }
      __syncthreads();
      if (!undecided) break;
    }
    if (threadIdx.x == 0) {
      const bool bad = !(t <= tol * tol);  // NaN counts as bad
      flag[b] = bad ? 1 : 0;
      if (bad && count) atomicAdd(count, 1);
    }
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

// Register-blocked FP32 Gauss-Jordan for 64 < n <= 128 (blocks padded to 128 with the
// identity).  Warp w owns columns 8w..8w+7, lane l owns rows 4l..4l+3: 32 complex
// entries per thread stay in registers for the whole elimination.  Pivoting is implicit
// (no row swaps): step k picks the unused row p with the largest |re|+|im| in column k
// (warp-local search in the warp owning column k), and at the end the inverse is
// X[k][j] = M[P[k]][P^-1[j]].  One __syncthreads per step (pivot column and index are
// double-buffered in shared memory).  Lookahead: during step k the warp owning column k+1
// first forms that column's step-k values (the same FMAs as its update) and takes step
// k+1's pivot, so the search overlaps the other warps' updates.
template <typename TC>
__global__ __launch_bounds__(512, 1) void zinv_f32_rb_kernel(InvArgs a) {
  __shared__ float2 colbuf[2][128];
  __shared__ int pbuf[2];
  __shared__ int perm[128], pinv[128];
  __shared__ int badflag;
  const int n = a.n;
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  for (long long b = blockIdx.x; b < a.batch; b += gridDim.x) {
    if (a.active && !a.active[b]) continue;
    const TC* A = batch_ptr<const TC>(a.A, b);
    TC* X = batch_ptr<TC>(a.X, b);
    const int lda = a.A.ld, ld = a.X.ld;
    float2 M[4][8];
#pragma unroll
    for (int rr = 0; rr < 4; ++rr)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int r = 4 * l + rr, c = 8 * w + j;
        if (r < n && c < n) M[rr][j] = to_f2(A[r + (long long)c * lda]);
        else M[rr][j] = make_float2(r == c ? 1.f : 0.f, 0.f);
      }
    unsigned used = 0;
    if (tid == 0) badflag = 0;
    // pivot search over one column (this lane's rows in v) into buffer slot qq: the unused
    // row with the largest |re|+|im|, the lowest row on ties
    auto search = [&](const float2 (&v)[4], int qq) {
      float best = -1.f;
      int bi = 0x7fffffff;
#pragma unroll
      for (int rr = 0; rr < 4; ++rr) {
        colbuf[qq][4 * l + rr] = v[rr];
        float m = fabsf(v[rr].x) + fabsf(v[rr].y);
        if (!(m == m)) m = 0.f;  // NaN: still selectable (flagged below), never skipped
        if (!((used >> rr) & 1u) && (m > best || (m == best && 4 * l + rr < bi))) {
          best = m;
          bi = 4 * l + rr;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (bi > 127) bi = 0;  // unreachable: 128 - k >= 1 unused rows always compete
      if (l == 0) {
        pbuf[qq] = bi;
        if (!(best > 0.f) || !isfinite(best)) badflag = 1;
      }
    };
    if (w == 0) {  // step 0's pivot: column 0 as loaded
      float2 v[4];
#pragma unroll
      for (int rr = 0; rr < 4; ++rr) v[rr] = M[rr][0];
      search(v, 0);
    }
    __syncthreads();
    for (int k = 0; k < 128; ++k) {
      const int q = k & 1, wk = k >> 3, ck = k & 7;
      const int p = pbuf[q];
      const int lp = p >> 2, rp = p & 3;
      const float2 piv = colbuf[q][p];
      const float d = piv.x * piv.x + piv.y * piv.y;
      const float2 inv = d > 0.f ? make_float2(piv.x / d, -piv.y / d) : make_float2(0.f, 0.f);
      // pivot row (my 8 columns), broadcast from the owning lane, normalised
      float2 rowp[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float2 v;
        v.x = (rp == 0) ? M[0][j].x : (rp == 1) ? M[1][j].x : (rp == 2) ? M[2][j].x : M[3][j].x;
        v.y = (rp == 0) ? M[0][j].y : (rp == 1) ? M[1][j].y : (rp == 2) ? M[2][j].y : M[3][j].y;
        v.x = __shfl_sync(0xffffffffu, v.x, lp);
        v.y = __shfl_sync(0xffffffffu, v.y, lp);
        rowp[j] = make_float2(v.x * inv.x - v.y * inv.y, v.x * inv.y + v.y * inv.x);
        if (w == wk && j == ck) rowp[j] = inv;
      }
      if (l == lp) used |= 1u << rp;
      if (k < 127 && w == ((k + 1) >> 3)) {
        // lookahead: column k+1 after step k (row p: the normalised pivot row; the others:
        // the update below), then step k+1's pivot into the other buffer slot
        const int cn = (k + 1) & 7;
        float2 rn = rowp[0];
#pragma unroll
        for (int j = 1; j < 8; ++j)
          if (j == cn) rn = rowp[j];
        float2 v[4];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
          float2 m = M[rr][0];
#pragma unroll
          for (int j = 1; j < 8; ++j)
            if (j == cn) m = M[rr][j];
          if (4 * l + rr == p) {
            v[rr] = rn;
          } else {
            const float2 f = colbuf[q][4 * l + rr];
            m.x = fmaf(-f.x, rn.x, m.x); m.x = fmaf(f.y, rn.y, m.x);
            m.y = fmaf(-f.x, rn.y, m.y); m.y = fmaf(-f.y, rn.x, m.y);
            v[rr] = m;
          }
        }
        search(v, q ^ 1);
      }
      // the pivot column's special case only exists in warp wk: the other warps run the
      // update without testing for it (same arithmetic in both)
      if (w == wk) {
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
          const int r = 4 * l + rr;
          if (r == p) {
#pragma unroll
            for (int j = 0; j < 8; ++j) M[rr][j] = rowp[j];
          } else {
            const float2 f = colbuf[q][r];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              if (j == ck) {
                M[rr][j] = make_float2(-(f.x * inv.x - f.y * inv.y), -(f.x * inv.y + f.y * inv.x));
              } else {
                float2 m = M[rr][j];
                m.x = fmaf(-f.x, rowp[j].x, m.x); m.x = fmaf(f.y, rowp[j].y, m.x);
                m.y = fmaf(-f.x, rowp[j].y, m.y); m.y = fmaf(-f.y, rowp[j].x, m.y);
                M[rr][j] = m;
              }
            }
          }
        }
      } else {
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
          const int r = 4 * l + rr;
          if (r == p) {
#pragma unroll
            for (int j = 0; j < 8; ++j) M[rr][j] = rowp[j];
          } else {
            const float2 f = colbuf[q][r];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              float2 m = M[rr][j];
              m.x = fmaf(-f.x, rowp[j].x, m.x); m.x = fmaf(f.y, rowp[j].y, m.x);
              m.y = fmaf(-f.x, rowp[j].y, m.y); m.y = fmaf(-f.y, rowp[j].x, m.y);
              M[rr][j] = m;
            }
          }
        }
      }
      if (tid == 0) perm[k] = p;
      __syncthreads();
    }
    __syncthreads();
    if (tid < 128) pinv[tid] = -1;
    __syncthreads();
    if (tid < 128) pinv[perm[tid] & 127] = tid;
    __syncthreads();
#pragma unroll
    for (int rr = 0; rr < 4; ++rr)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int orow = pinv[4 * l + rr], ocol = perm[8 * w + j];
        if (orow >= 0 && orow < n && ocol >= 0 && ocol < n)
          X[orow + (long long)ocol * ld] = from_f2<TC>(M[rr][j]);
      }
    if (tid == 0 && badflag && a.status) atomicOr(&a.status[b], PT_SINGULAR);
    __syncthreads();
  }
}

long long grid_for(long long batch) { return batch < 65535 * 4 ? batch : 65535 * 4; }

}  // namespace

cudaError_t zinv_f64(const InvArgs& a, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  const size_t sm = (size_t)a.n * 2 * sizeof(cd) + (size_t)a.n * sizeof(int);
  zinv_f64_kernel<double2><<<(unsigned)grid_for(a.batch), NT64, sm, s>>>(a, nullptr, 0);
  count_launch();
  return cudaGetLastError();
}

template <typename TC>
cudaError_t zinv_f64_ws(const InvArgs& a, cd* W, long long wst, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (sizeof(TC) != 16 && !W) return cudaErrorInvalidValue;
  const size_t sm = (size_t)a.n * 2 * sizeof(cd) + (size_t)a.n * sizeof(int);
  zinv_f64_kernel<TC><<<(unsigned)grid_for(a.batch), NT64, sm, s>>>(a, W, wst);
  count_launch();
  return cudaGetLastError();
}
template cudaError_t zinv_f64_ws<double2>(const InvArgs&, cd*, long long, cudaStream_t);
template cudaError_t zinv_f64_ws<float2>(const InvArgs&, cd*, long long, cudaStream_t);

template <typename TC>
cudaError_t zinv_guard(int n, long long batch, BatchRef R, const unsigned char* active,
                       double tol, unsigned char* flag, int* count, cudaStream_t s) {
  if (batch <= 0) return cudaSuccess;
  zinv_guard_kernel<TC><<<(unsigned)grid_for(batch), 256, 0, s>>>(n, batch, R, active, tol, flag,
                                                                  count);
  count_launch();
  return cudaGetLastError();
}
template cudaError_t zinv_guard<double2>(int, long long, BatchRef, const unsigned char*, double,
                                         unsigned char*, int*, cudaStream_t);
template cudaError_t zinv_guard<float2>(int, long long, BatchRef, const unsigned char*, double,
                                        unsigned char*, int*, cudaStream_t);

template <typename TC>
cudaError_t zinv_f32(const InvArgs& a, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (a.n > 128) return cudaErrorInvalidValue;
  if (a.n > 64) {  // register-blocked elimination
    zinv_f32_rb_kernel<TC><<<(unsigned)grid_for(a.batch), 512, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
  }
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
