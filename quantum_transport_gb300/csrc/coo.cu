// Device Hamiltonian blocks from a COO matrix on the GPU.
//
// Restates the blocksize branch of devH_build_fromCOOfile
// (src/deviceHam_mod.f90:168-224).  The reference walks the entries in file
// order; for entry e = (row, col, h) with (ix, mm) = divmod(row, bs) and
// nn = col - ix*bs (0-based):
//
//   0 <= nn < bs:      Hii(ix)[mm, nn] = h; Hii(ix)[nn, mm] = conj(h);
//                      Sii(ix)[mm, nn] = s (when an overlap is given)
//   bs <= nn < 2 bs:   H1i(ix)[mm, nn - bs] = h
//
// and otherwise drops the entry (also when ix >= nx); then H1i(nx+1) = H1i(nx)
// and, without an overlap, Sii = I.  Later writes win.  The reference's own
// slab/local arithmetic works on the 1-based row and puts every slab's last
// orbital at local index 0, outside the block; this builder uses the 0-based
// divmod throughout, which agrees with the reference wherever the reference
// stays inside its arrays.
//
// GPU form, deterministic and bit-exact against that serial order:
//   1. per entry: each target element takes atomicMax of the key
//      2*e + t + 1 (t = 1 for the conjugate-transposed write, which comes
//      second within an entry);
//   2. per output element: read the winning key and gather that entry's
//      value (conjugated when t = 1); untouched elements are 0.
// Outputs are column-major bs x bs blocks, written once and coalesced.
#include "qt_abi.h"
#include "qt_kernels.h"

namespace qt {
namespace {

struct CooArgs {
  int nx, bs, base;
  long long nnz;
  const int* row;
  const int* col;
  const double2* h;
  const double2* s;               // nullable
  unsigned long long* kH;         // [nx][bs*bs] winning key per Hii element
  unsigned long long* k1;         // [nx][bs*bs] per H1i element
  unsigned long long* kS;         // [nx][bs*bs] per Sii element (with s)
  double2* Hii;                   // [nx][bs*bs]
  double2* H1i;                   // [nx+1][bs*bs]
  double2* Sii;                   // [nx][bs*bs]
};

__global__ void coo_claim_kernel(CooArgs a) {
  const long long per = (long long)a.bs * a.bs;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < a.nnz;
       e += (long long)gridDim.x * blockDim.x) {
    const long long r = (long long)a.row[e] - a.base, c = (long long)a.col[e] - a.base;
    if (r < 0 || c < 0) continue;
    const long long ix = r / a.bs, mm = r % a.bs;
    if (ix >= a.nx) continue;
    const long long nn = c - ix * a.bs;
    const unsigned long long key = 2ull * (unsigned long long)e + 1ull;
    if (nn >= 0 && nn < a.bs) {
      atomicMax(a.kH + ix * per + mm + a.bs * nn, key);
      atomicMax(a.kH + ix * per + nn + a.bs * mm, key + 1ull);
      if (a.s) atomicMax(a.kS + ix * per + mm + a.bs * nn, key);
    } else if (nn >= a.bs && nn < 2LL * a.bs) {
      atomicMax(a.k1 + ix * per + mm + a.bs * (nn - a.bs), key);
    }
  }
}

__device__ __forceinline__ double2 pick(const double2* v, unsigned long long key) {
  if (key == 0ull) return make_double2(0.0, 0.0);
  const unsigned long long k = key - 1ull;
  double2 x = v[k >> 1];
  if (k & 1ull) x.y = -x.y;
  return x;
}

__global__ void coo_gather_kernel(CooArgs a) {
  const long long per = (long long)a.bs * a.bs, total = per * (a.nx + 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long ix = t / per, el = t % per;
    // H1i(nx+1) = H1i(nx): the last coupling block repeats the one before it
    const long long src = ix < a.nx ? t : (a.nx - 1) * per + el;
    a.H1i[t] = pick(a.h, a.k1[src]);
    if (ix < a.nx) {
      a.Hii[t] = pick(a.h, a.kH[t]);
      if (a.s) {
        a.Sii[t] = pick(a.s, a.kS[t]);
      } else {
        const bool diag = (el % a.bs) == (el / a.bs);
        a.Sii[t] = make_double2(diag ? 1.0 : 0.0, 0.0);
      }
    }
  }
}

inline unsigned grid_for(long long n) {
  const long long g = (n + 255) / 256;
  return (unsigned)(g < 1 ? 1 : (g < 152LL * 64 ? g : 152LL * 64));
}

}  // namespace
}  // namespace qt

extern "C" qt_status qt_coo_blocks(qt_ctx* ctx, int nx, int bs, long long nnz, const int* row,
                                   const int* col, int index_base, const double* h,
                                   const double* s, double* Hii, double* H1i, double* Sii,
                                   unsigned flags) {
  if (!ctx || nx <= 0 || bs <= 0 || nnz < 0 || !Hii || !H1i || !Sii)
    QT_FAIL(QT_ERR_ARG, "bad COO block arguments");
  if (nnz > 0 && (!row || !col || !h)) QT_FAIL(QT_ERR_ARG, "COO entries missing");
  if (index_base != 0 && index_base != 1) QT_FAIL(QT_ERR_ARG, "index_base must be 0 or 1");
  if (nnz >= (1LL << 62)) QT_FAIL(QT_ERR_ARG, "too many COO entries");
  cudaSetDevice(qt::ctx_device(ctx));
  cudaStream_t st = qt::ctx_stream(ctx);
  const long long per = (long long)bs * bs;
  const size_t nblk = (size_t)nx * per, out1 = nblk + (size_t)per;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  const bool has_s = s != nullptr;

  size_t bytes = 3 * nblk * 8 + 1024;  // keys
  if (!devp) bytes += (size_t)nnz * (8 + 16 * (has_s ? 2 : 1)) + (2 * nblk + out1) * 16 + 2048;
  void* stage = nullptr;
  QT_CUDA_TRY(cudaMallocAsync(&stage, bytes, st));
  char* p = static_cast<char*>(stage);
  auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };

  qt::CooArgs a{};
  a.nx = nx; a.bs = bs; a.base = index_base; a.nnz = nnz;
  a.kH = reinterpret_cast<unsigned long long*>(take(nblk * 8));
  a.k1 = reinterpret_cast<unsigned long long*>(take(nblk * 8));
  a.kS = reinterpret_cast<unsigned long long*>(take(nblk * 8));
  if (devp) {
    a.row = row; a.col = col;
    a.h = reinterpret_cast<const double2*>(h);
    a.s = reinterpret_cast<const double2*>(s);
    a.Hii = reinterpret_cast<double2*>(Hii);
    a.H1i = reinterpret_cast<double2*>(H1i);
    a.Sii = reinterpret_cast<double2*>(Sii);
  } else {
    int* drow = reinterpret_cast<int*>(take((size_t)nnz * 4));
    int* dcol = reinterpret_cast<int*>(take((size_t)nnz * 4));
    double2* dh = reinterpret_cast<double2*>(take((size_t)nnz * 16));
    double2* ds = has_s ? reinterpret_cast<double2*>(take((size_t)nnz * 16)) : nullptr;
    a.Hii = reinterpret_cast<double2*>(take(nblk * 16));
    a.H1i = reinterpret_cast<double2*>(take(out1 * 16));
    a.Sii = reinterpret_cast<double2*>(take(nblk * 16));
    if (nnz > 0) {
      cudaMemcpyAsync(drow, row, (size_t)nnz * 4, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(dcol, col, (size_t)nnz * 4, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(dh, h, (size_t)nnz * 16, cudaMemcpyHostToDevice, st);
      if (has_s) cudaMemcpyAsync(ds, s, (size_t)nnz * 16, cudaMemcpyHostToDevice, st);
    }
    a.row = drow; a.col = dcol; a.h = dh; a.s = ds;
  }
  // the three key arrays were taken first and back to back
  const size_t kspan = (size_t)(reinterpret_cast<char*>(a.kS + nblk) - reinterpret_cast<char*>(a.kH));
  cudaMemsetAsync(a.kH, 0, kspan, st);
  if (nnz > 0) {
    qt::coo_claim_kernel<<<qt::grid_for(nnz), 256, 0, st>>>(a);
    qt::count_launch();
  }
  qt::coo_gather_kernel<<<qt::grid_for((long long)out1), 256, 0, st>>>(a);
  qt::count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFreeAsync(stage, st);
    QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  }
  if (!devp) {
    cudaMemcpyAsync(Hii, a.Hii, nblk * 16, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(H1i, a.H1i, out1 * 16, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(Sii, a.Sii, nblk * 16, cudaMemcpyDeviceToHost, st);
  }
  cudaFreeAsync(stage, st);
  if (!devp || (flags & QT_FLAG_SYNC)) QT_CUDA_TRY(cudaStreamSynchronize(st));
  return QT_OK;
}
