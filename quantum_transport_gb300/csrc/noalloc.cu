// Allocation-free variant of the split-precision block product (qt_zgemm_batch_noalloc).
//
// The split product needs scratch beyond its inputs and outputs: a table of
// 256 scale exponents per batch entry, written by its prologue kernel and read
// by the tensor-core kernel.  qt_zgemm_batch takes that table from the
// context's device arena, which it grows with cudaMalloc on demand.  Some
// callers cannot allocate device memory:
//   * hosts whose device memory is owned by another allocator -- a framework's
//     caching pool, or a Fortran code whose buffers live in OpenMP
//     `target enter data` regions (as the reference's cuda_rgf_init does);
//   * latency-critical loops, where cudaMalloc/cudaFree would implicitly
//     synchronise the whole device and stall the other streams.
// For them this entry point keeps the table in a file-scope device array of
// fixed size and needs no context: it allocates nothing and takes the caller's
// stream.
//
// Limits and sharing rules:
//   * at most QT_NOALLOC_MAX_BATCH (512) batch entries per call: 512 x 256
//     ints = 512 KiB of device memory, held by every GPU that loads the library
//     until the process exits;
//   * the array belongs to the library's device module.  Under CUDA's default
//     lazy module loading that module is loaded by the first call on a device,
//     which can allocate module memory and synchronise: make one warm-up call
//     outside latency-critical regions and before any stream capture (or set
//     CUDA_MODULE_LOADING=EAGER);
//   * every call looks up the array's device address (cudaGetSymbolAddress,
//     with the caller's device current), so the address stays valid across a
//     device reset;
//   * every call shares the one array: calls that overlap on the GPU (other
//     streams, other host threads) race on it.  Serialise them, e.g. on one
//     stream.  The exponent table needs no clearing between calls: the prologue
//     rewrites every exponent the product then reads;
//   * a wait inside the tensor-core kernel that runs out (4 s) leaves C partly
//     written.  Such timeouts are counted in a word of the same array, never in
//     the context library's counter; qt_noalloc_timeouts reads and clears it
//     after the caller has synchronised its stream.
#include "../../include/qt_rgf.h"
#include "qt_common.cuh"
#include "qt_kernels.h"

namespace {

// [0, MAX * 256): exponent table; [MAX * 256]: timeout count of the tensor-core kernel
constexpr int kTimeoutWord = QT_NOALLOC_MAX_BATCH * 256;
static __device__ __align__(256) int g_noalloc_scratch[kTimeoutWord + 64];

// device address of the array on the current device (host code only sees a stand-in)
cudaError_t scratch_address(int** out) {
  return cudaGetSymbolAddress(reinterpret_cast<void**>(out), g_noalloc_scratch);
}

int parse_op(char c) {
  if (c == 'N' || c == 'n') return qt::OP_N;
  if (c == 'C' || c == 'c') return qt::OP_C;
  return -1;
}

}  // namespace

extern "C" qt_status qt_zgemm_batch_noalloc(int n, int batch, char opA, const double* A,
                                            int64_t a_stride, char opB, const double* B,
                                            int64_t b_stride, const double* alpha,
                                            const double* beta, const double* D,
                                            int64_t d_stride, double* C, int64_t c_stride,
                                            int slices, void* stream) {
  const int oa = parse_op(opA), ob = parse_op(opB);
  if (!A || !B || !C || n <= 0 || n > 128 || batch <= 0 || oa < 0 || ob < 0) {
    qt_set_last_error("qt_zgemm_batch_noalloc: need device pointers, 0 < n <= 128, op in {N, C}",
                      __FILE__, __LINE__);
    return QT_ERR_ARG;
  }
  if (batch > QT_NOALLOC_MAX_BATCH) {
    qt_set_last_error("qt_zgemm_batch_noalloc: batch exceeds QT_NOALLOC_MAX_BATCH (512), the size "
                      "of its static scratch; split the call",
                      __FILE__, __LINE__);
    return QT_ERR_ARG;
  }
  const int sl = slices ? slices : 4;
  if (sl != 4 && sl != 6 && sl != 7) {
    qt_set_last_error("qt_zgemm_batch_noalloc: slices must be 0 (4), 4, 6 or 7", __FILE__,
                      __LINE__);
    return QT_ERR_ARG;
  }
  if ((alpha && alpha[1] != 0.0) || (beta && beta[1] != 0.0)) {
    qt_set_last_error("qt_zgemm_batch_noalloc: alpha and beta must be real", __FILE__, __LINE__);
    return QT_ERR_UNSUPPORTED;
  }
  int* scales = nullptr;
  cudaError_t e = scratch_address(&scales);
  if (e != cudaSuccess) {
    qt_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return QT_ERR_CUDA;
  }
  qt::GemmArgs g{};
  g.m = g.n = g.k = n;
  auto ref = [](const void* p, long long stride, int ld) {
    qt::BatchRef r{};
    r.p = const_cast<void*>(p);
    r.stride = stride;
    r.ld = ld;
    return r;
  };
  g.A = ref(A, a_stride, n);
  g.B = ref(B, b_stride, n);
  g.C = ref(C, c_stride, n);
  g.D = D ? ref(D, d_stride, n) : ref(nullptr, 0, 1);
  g.Z = ref(nullptr, 0, 1);
  g.opA = oa;
  g.opB = ob;
  g.alpha_re = alpha ? alpha[0] : 1.0;
  g.beta_re = beta ? beta[0] : 0.0;
  g.batch = batch;
  g.active = nullptr;
  g.scales = scales;
  g.timeouts = scales + kTimeoutWord;
  e = qt::zgemm_oz(g, sl, sl - 1, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    qt_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return QT_ERR_CUDA;
  }
  return QT_OK;
}

extern "C" qt_status qt_noalloc_timeouts(int* count, void* stream) {
  if (!count) {
    qt_set_last_error("qt_noalloc_timeouts: count is null", __FILE__, __LINE__);
    return QT_ERR_ARG;
  }
  int* base = nullptr;
  cudaError_t e = scratch_address(&base);
  const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, base + kTimeoutWord, sizeof(int),
                                            cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && h) e = cudaMemsetAsync(base + kTimeoutWord, 0, sizeof(int), s);
  if (e == cudaSuccess && h) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    qt_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return QT_ERR_CUDA;
  }
  *count = h;
  return QT_OK;
}
