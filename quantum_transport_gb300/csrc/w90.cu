// Slab blocks of a Wannier90 tight-binding model on the GPU, for many transverse
// k-points in one launch: the device Hamiltonian the RGF sweep consumes.
//
// Restates w90_MAT_DEF (src/wannierHam3d.f90:273-301).  For a slab of ns cells
// of nb orbitals, with cells i, k = 0..ns-1 and d = i - k:
//
//   H_ii(k)[i, k]     = sum_{Ry, Rz} Hr(:, :, d,      Ry, Rz) exp(-i r.kv)
//   H_{i+1,i}(k)[i,k] = sum_{Ry, Rz} Hr(:, :, d + ns, Ry, Rz) exp(-i r.kv)
//   r = d alpha + Ry beta + Rz gamm
//
// where a term exists only if its Rx lies in the model's range.  As in the
// reference, the phase of the coupling block uses r without the ns alpha shift.
// One thread per output element (both blocks): the sum over Ry, Rz runs in FP64
// with sincos for the phase.
#include <math.h>

#include "qt_abi.h"
#include "qt_kernels.h"

namespace qt {
namespace {

struct W90Args {
  int nb, ns, nk;
  int xmin, xmax, ymin, ymax, zmin, zmax;
  const double2* Hr;  // Fortran Hr(nb, nb, nxr, nyr, nzr)
  double alpha[3], beta[3], gamm[3];
  const double* kv;  // [nk][3] Cartesian k vectors
  double2* H00;      // [nk][nm*nm] column-major
  double2* H10;
};

__global__ void w90_blocks_kernel(W90Args a) {
  const int nm = a.nb * a.ns;
  const long long per = (long long)nm * nm, total = per * a.nk;
  const int nxr = a.xmax - a.xmin + 1, nyr = a.ymax - a.ymin + 1;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long ik = t / per, e = t % per;
    const int row = (int)(e % nm), col = (int)(e / nm);
    const int i = row / a.nb, m = row % a.nb, k = col / a.nb, n = col % a.nb;
    const int d = i - k;
    const double* kv = a.kv + 3 * ik;
    const bool in00 = d >= a.xmin && d <= a.xmax;
    const bool in10 = d + a.ns >= a.xmin && d + a.ns <= a.xmax;
    double2 h00 = make_double2(0.0, 0.0), h10 = h00;
    if (in00 || in10) {
      for (int jy = a.ymin; jy <= a.ymax; ++jy) {
        for (int lz = a.zmin; lz <= a.zmax; ++lz) {
          double rk = 0.0;
#pragma unroll
          for (int c = 0; c < 3; ++c)
            rk += (d * a.alpha[c] + jy * a.beta[c] + lz * a.gamm[c]) * kv[c];
          double sn, cs;
          sincos(-rk, &sn, &cs);
          const long long yz = (long long)(jy - a.ymin) + (long long)nyr * (lz - a.zmin);
          if (in00) {
            const double2 h = a.Hr[m + (long long)a.nb * (n + (long long)a.nb *
                                                          ((d - a.xmin) + (long long)nxr * yz))];
            h00.x += h.x * cs - h.y * sn;
            h00.y += h.x * sn + h.y * cs;
          }
          if (in10) {
            const double2 h = a.Hr[m + (long long)a.nb * (n + (long long)a.nb *
                                                          ((d + a.ns - a.xmin) + (long long)nxr * yz))];
            h10.x += h.x * cs - h.y * sn;
            h10.y += h.x * sn + h.y * cs;
          }
        }
      }
    }
    a.H00[t] = h00;
    a.H10[t] = h10;
  }
}

}  // namespace
}  // namespace qt

extern "C" qt_status qt_w90_blocks(qt_ctx* ctx, int nb, int ns, const int* range,
                                   const double* Hr, const double* cell, int nk,
                                   const double* kvec, double* H00, double* H10,
                                   unsigned flags) {
  if (!ctx || !range || !Hr || !cell || !kvec || !H00 || !H10 || nb <= 0 || ns <= 0 || nk <= 0)
    QT_FAIL(QT_ERR_ARG, "bad w90 block arguments");
  if (range[0] > range[1] || range[2] > range[3] || range[4] > range[5])
    QT_FAIL(QT_ERR_ARG, "w90 R ranges must satisfy min <= max");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t s = qt::ctx_stream(ctx);
  qt::W90Args a{};
  a.nb = nb; a.ns = ns; a.nk = nk;
  a.xmin = range[0]; a.xmax = range[1];
  a.ymin = range[2]; a.ymax = range[3];
  a.zmin = range[4]; a.zmax = range[5];
  for (int c = 0; c < 3; ++c) {
    a.alpha[c] = cell[c];
    a.beta[c] = cell[3 + c];
    a.gamm[c] = cell[6 + c];
  }
  const long long nr = (long long)(range[1] - range[0] + 1) * (range[3] - range[2] + 1) *
                       (range[5] - range[4] + 1);
  const long long hr_n = (long long)nb * nb * nr;
  const long long nm = (long long)nb * ns, out_n = (long long)nk * nm * nm;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  void* stage = nullptr;
  if (devp) {
    a.Hr = reinterpret_cast<const double2*>(Hr);
    a.kv = kvec;
    a.H00 = reinterpret_cast<double2*>(H00);
    a.H10 = reinterpret_cast<double2*>(H10);
  } else {
    const size_t bytes = (size_t)hr_n * 16 + (size_t)nk * 24 + 2 * (size_t)out_n * 16 + 1024;
    QT_CUDA_TRY(cudaMallocAsync(&stage, bytes, s));
    char* p = static_cast<char*>(stage);
    auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
    double2* hr = reinterpret_cast<double2*>(take((size_t)hr_n * 16));
    double* kv = reinterpret_cast<double*>(take((size_t)nk * 24));
    a.H00 = reinterpret_cast<double2*>(take((size_t)out_n * 16));
    a.H10 = reinterpret_cast<double2*>(take((size_t)out_n * 16));
    cudaMemcpyAsync(hr, Hr, (size_t)hr_n * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(kv, kvec, (size_t)nk * 24, cudaMemcpyHostToDevice, s);
    a.Hr = hr;
    a.kv = kv;
  }
  const long long g = (out_n + 255) / 256;
  qt::w90_blocks_kernel<<<(unsigned)(g < 65535LL * 16 ? g : 65535LL * 16), 256, 0, s>>>(a);
  qt::count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  if (!devp) {
    cudaMemcpyAsync(H00, a.H00, (size_t)out_n * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(H10, a.H10, (size_t)out_n * 16, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(stage, s);
    QT_CUDA_TRY(cudaStreamSynchronize(s));
  } else if (flags & QT_FLAG_SYNC) {
    QT_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return QT_OK;
}
