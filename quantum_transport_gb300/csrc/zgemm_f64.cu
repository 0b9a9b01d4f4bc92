// Batched complex128 GEMM on the FP64 pipes (plain-FP64 path).
//
//   C_b = alpha * op(A_b) * op(B_b) + beta * D_b + diag(z_b)
//
// op in {N, C (conjugate transpose), T}.  This is the batched replacement of
// the reference's zgemm calls (src/cuda_rgf_mod.f90:152-175, 293-370 through
// cuBLAS; src/matrix_c.f90:615-660 MUL_C on the CPU).  One CTA computes a
// 64x64 tile of one batch entry with 256 threads, 4x4 complex outputs per
// thread, K staged through shared memory in steps of 8.  GB300's FP64 rate is
// the bound for this kernel; it exists as the plain-FP64 baseline and parity
// anchor for the split-precision tensor-core path.
#include "qt_common.cuh"
#include "qt_kernels.h"

namespace qt {

namespace {

constexpr int BM = 64, BN = 64, BK = 8, NT = 256;

__device__ __forceinline__ cd load_op(const cd* M, int ld, int op, int r, int c) {
  // element (r, c) of op(M), M column-major with leading dimension ld
  if (op == OP_N) return M[r + (long long)c * ld];
  cd v = M[c + (long long)r * ld];
  return op == OP_C ? cconj(v) : v;
}

__global__ __launch_bounds__(NT) void zgemm_f64_kernel(GemmArgs a) {
  __shared__ cd As[BK][BM];
  __shared__ cd Bs[BK][BN];
  const int tiles_m = (a.m + BM - 1) / BM;
  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  const int m0 = tm * BM, n0 = tn * BN;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  for (long long b = blockIdx.y; b < a.batch; b += gridDim.y) {
    if (a.active && !a.active[b]) continue;
    const cd* A = batch_ptr<const cd>(a.A, b);
    const cd* B = batch_ptr<const cd>(a.B, b);
    cd acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = cd{0.0, 0.0};
    for (int k0 = 0; k0 < a.k; k0 += BK) {
      for (int e = tid; e < BM * BK; e += NT) {
        int i, kk;
        if (a.opA == OP_N) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
        const int gi = m0 + i, gk = k0 + kk;
        As[kk][i] = (gi < a.m && gk < a.k) ? load_op(A, a.A.ld, a.opA, gi, gk) : cd{0.0, 0.0};
      }
      for (int e = tid; e < BK * BN; e += NT) {
        int j, kk;
        if (a.opB == OP_N) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
        const int gj = n0 + j, gk = k0 + kk;
        Bs[kk][j] = (gj < a.n && gk < a.k) ? load_op(B, a.B.ld, a.opB, gk, gj) : cd{0.0, 0.0};
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        cd av[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) cfma(acc[i][j], av[i], bv[j]);
      }
      __syncthreads();
    }
    cd* C = batch_ptr<cd>(a.C, b);
    const cd* D = a.D.p ? batch_ptr<const cd>(a.D, b) : nullptr;
    cd z = {0.0, 0.0};
    if (a.Z.p) z = *batch_ptr<const cd>(a.Z, b);
    const cd alpha = {a.alpha_re, a.alpha_im}, beta = {a.beta_re, a.beta_im};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gi = m0 + ty + 16 * i;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int gj = n0 + tx + 16 * j;
        if (gi < a.m && gj < a.n) {
          cd v = cmul(alpha, acc[i][j]);
          if (D) v = cadd(v, cmul(beta, D[gi + (long long)gj * a.D.ld]));
          if (gi == gj) v = cadd(v, z);
          C[gi + (long long)gj * a.C.ld] = v;
        }
      }
    }
  }
}

}  // namespace

cudaError_t zgemm_f64(const GemmArgs& a, cudaStream_t s) {
  if (a.batch <= 0 || a.m <= 0 || a.n <= 0) return cudaSuccess;
  const int tiles = ((a.m + BM - 1) / BM) * ((a.n + BN - 1) / BN);
  const long long by = a.batch < 65535 ? a.batch : 65535;
  zgemm_f64_kernel<<<dim3(tiles, (unsigned)by), NT, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace qt
