// Shared device/host helpers for the batched RGF kernels (sm_103a).
//
// Storage convention everywhere: an n x n block is complex128 column-major,
// element (i,j) at p[i + j*ld], interleaved (re, im) doubles -- the memory
// image of the reference's Fortran complex(8) arrays (src/matrix_c.f90:34-39).
// A batch of blocks is addressed per batch index b through a "BatchRef":
// p + (b % mod) * stride (mod == 0 means "no modulus").  This lets one kernel
// read per-point data (stride = n*n), data shared by all points (stride = 0)
// and per-k data for points ordered (E-major, k-minor) (mod = nk).
#pragma once
#include <cuda_runtime.h>
#include <cuComplex.h>
#include <stdint.h>

namespace qt {

struct BatchRef {
  void* p;
  long long stride;  // elements (complex) between consecutive batch entries
  int mod;           // 0: none; else batch index is taken modulo mod
  int ld;            // leading dimension (elements)
  // Optional indirection: when idx != nullptr, the batch entry is idx[b].
  const int* idx;
};

__host__ __device__ inline long long batch_index(const BatchRef& r, long long b) {
  long long e = r.idx ? (long long)r.idx[b] : b;
  if (r.mod > 0) e %= r.mod;
  return e;
}

template <typename T>
__host__ __device__ inline T* batch_ptr(const BatchRef& r, long long b) {
  return reinterpret_cast<T*>(r.p) + batch_index(r, b) * r.stride;
}

// complex helpers (double)
struct cd {
  double x, y;
};
__device__ __forceinline__ cd cmake(double a, double b) { return cd{a, b}; }
__device__ __forceinline__ cd cadd(cd a, cd b) { return cd{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cd csub(cd a, cd b) { return cd{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cd cmul(cd a, cd b) { return cd{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd cconj(cd a) { return cd{a.x, -a.y}; }
// acc += a*b
__device__ __forceinline__ void cfma(cd& acc, cd a, cd b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ cd cload(const void* base, long long off) {
  const double2 v = reinterpret_cast<const double2*>(base)[off];
  return cd{v.x, v.y};
}
__device__ __forceinline__ void cstore(void* base, long long off, cd v) {
  reinterpret_cast<double2*>(base)[off] = make_double2(v.x, v.y);
}

// Per-point status bits (also exported through include/qt_rgf.h).
enum : int {
  PT_OK = 0,
  PT_SINGULAR = 1,
  PT_SANCHO_NOT_CONVERGED = 2,
  PT_NONFINITE = 4,
};

}  // namespace qt

#define QT_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) {                                \
      qt_set_last_error(cudaGetErrorString(_e), __FILE__, __LINE__); \
      return QT_ERR_CUDA;                                   \
    }                                                       \
  } while (0)

extern "C" void qt_set_last_error(const char* msg, const char* file, int line);
