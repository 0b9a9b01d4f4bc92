// Multilayer perceptron of the learned SCBA mixing step: BF16 weights and
// activations, FP32 accumulation, trained with AdamW.  The reference has no
// counterpart (its SCBA loop mixes linearly, src/gw_mod.f90:747-749).
//
// Network: n_in -> width (GELU) -> ... (depth hidden layers) -> n_out, loss =
// mean squared error.  Every dense contraction -- forward, input gradient and
// weight gradient -- is one launch of mlp_gemm_kernel on the tcgen05 tensor
// cores:
//
//   C[m, n] = sum_k A(m, k) B(n, k)      A(m, k) = A[m*sam + k*sak]
//                                        B(n, k) = B[n*sbn + k*sbk]
//
// Operands are FP32 or BF16 in global memory, read with arbitrary strides so
// that the transposed products of the backward pass need no transposed copies.
// Producer warps round them to BF16 (round to nearest even) into the
// canonical K-major shared-memory layout.  The epilogue either stores FP32,
// adds the bias, or adds the bias and applies GELU (keeping the FP32
// pre-activation for the backward pass).
//
// Roles per CTA (288 threads): warps 0-3 epilogue (TMEM lanes 0-127), warps
// 4-7 producers, warp 8 TMEM allocation and the MMA-issuing thread.  Tile
// 128 x 128 (one FP32 accumulator of 128 TMEM columns), 64 K per stage.
// Every mbarrier wait is bounded (4 s) and counted in g_mlp_timeouts.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "qt_abi.h"
#include "qt_kernels.h"
#include "tc_ptx.cuh"

namespace qt {

__device__ int g_mlp_timeouts = 0;

namespace {

constexpr int KCH = 64;                          // K elements per pipeline stage
constexpr uint32_t M_LBO = 128;                  // K-adjacent core matrices
constexpr uint32_t M_SBO = (KCH / 8) * 128;      // consecutive 8-row groups
constexpr int TILE_BYTES = 128 * KCH * 2;        // one 128-row BF16 tile: 16 KB
constexpr int MLP_THREADS = 288;
constexpr int MLP_MMA_WARP = 8;
constexpr int MLP_PRODUCERS = 128;
constexpr uint64_t MLP_TIMEOUT_NS = 4000000000ull;

enum { EPI_STORE = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2 };

struct MlpGemm {
  int M, N, K;
  const void* A;
  long long sam, sak;
  const void* B;
  long long sbn, sbk;
  float* C;  // EPI_STORE, EPI_BIAS: FP32 output, C[m*scm + n*scn]
  long long scm, scn;
  float beta;  // EPI_STORE: C = acc + beta C (beta = 0 does not read C)
  int epi;
  const float* bias;  // [N]
  float* pre;         // EPI_BIAS_GELU: pre-activation [m*ldp + n]
  long long ldp;
  uint16_t* act;  // EPI_BIAS_GELU: GELU(pre) as BF16 [m*lda + n]
  long long lda;
};

// FP32 -> BF16 bits, round to nearest even (NaN kept quiet)
__host__ __device__ __forceinline__ uint16_t f2bf(float x) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
#endif
  if ((u & 0x7FFFFFFFu) > 0x7F800000u) return (uint16_t)((u >> 16) | 0x40u);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

template <typename T> __device__ __forceinline__ uint16_t load_bf(const void* p, long long i);
template <> __device__ __forceinline__ uint16_t load_bf<float>(const void* p, long long i) {
  return f2bf(reinterpret_cast<const float*>(p)[i]);
}
template <> __device__ __forceinline__ uint16_t load_bf<uint16_t>(const void* p, long long i) {
  return reinterpret_cast<const uint16_t*>(p)[i];
}

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// one 128-row x 64-K operand tile row `r` (global row `row`) into shared memory
template <typename T>
__device__ __forceinline__ void stage_row(unsigned char* tile, int r, int row, int nrows, int k0,
                                          int K, const void* P, long long srow, long long sk) {
  const bool in_row = row < nrows;
#pragma unroll
  for (int gq = 0; gq < KCH / 8; ++gq) {
    uint32_t w[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int ka = k0 + gq * 8 + 2 * h, kb = ka + 1;
      const uint16_t lo = (in_row && ka < K) ? load_bf<T>(P, row * srow + ka * sk) : (uint16_t)0;
      const uint16_t hi = (in_row && kb < K) ? load_bf<T>(P, row * srow + kb * sk) : (uint16_t)0;
      w[h] = (uint32_t)lo | ((uint32_t)hi << 16);
    }
    const uint32_t off = (uint32_t)((r >> 3) * M_SBO + gq * M_LBO + (r & 7) * 16);
    *reinterpret_cast<uint4*>(tile + off) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

template <typename TA, typename TB>
__global__ void __launch_bounds__(MLP_THREADS, 1) mlp_gemm_kernel(MlpGemm g, int stages) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int stage_bytes = 2 * TILE_BYTES;
  unsigned char* tiles = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)stages * stage_bytes);
  uint64_t* full = bars;
  uint64_t* empty = bars + stages;
  uint64_t* tmem_full = bars + 2 * stages;
  uint64_t* tmem_empty = tmem_full + 1;
  uint64_t* drain = tmem_full + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tmem_full + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = (g.M + 127) / 128, nt = (g.N + 127) / 128, nk = (g.K + KCH - 1) / KCH;
  const long long items = (long long)mt * nt;
  auto wait = [&](uint64_t* bar, uint32_t parity) {
    return tc::mbar_wait(bar, parity, abort_flag, &g_mlp_timeouts, MLP_TIMEOUT_NS);
  };

  if (tid == 0) {
    for (int s = 0; s < stages; ++s) {
      tc::mbar_init(&full[s], MLP_PRODUCERS);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(tmem_full, 1);
    tc::mbar_init(tmem_empty, 128);
    tc::mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MLP_MMA_WARP) tc::tmem_alloc(tmem_slot, 128);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp >= 4 && warp < 8) {
    // ======================== producers: thread p stages row p of the A and B tiles
    const int p = tid - 128;
    uint32_t gchunk = 0;
    for (long long w = blockIdx.x; w < items && !*abort_flag; w += gridDim.x) {
      const int m0 = (int)(w / nt) * 128, n0 = (int)(w % nt) * 128;
      for (int c = 0; c < nk; ++c, ++gchunk) {
        const int st = gchunk % stages;
        const uint32_t ph = (gchunk / stages) & 1;
        if (!wait(&empty[st], ph ^ 1)) break;
        unsigned char* sA = tiles + (size_t)st * stage_bytes;
        stage_row<TA>(sA, p, m0 + p, g.M, c * KCH, g.K, g.A, g.sam, g.sak);
        stage_row<TB>(sA + TILE_BYTES, p, n0 + p, g.N, c * KCH, g.K, g.B, g.sbn, g.sbk);
        tc::fence_proxy_async();
        tc::mbar_arrive(&full[st]);
      }
    }
  } else if (warp == MLP_MMA_WARP) {
    // ======================== MMA issuer (one thread)
    if (lane == 0) {
      const uint32_t idesc = tc::make_idesc(128, 128);
      uint32_t proc = 0, gchunk = 0;
      for (long long w = blockIdx.x; w < items && !*abort_flag; w += gridDim.x) {
        if (!wait(tmem_empty, (proc & 1) ^ 1)) break;
        tc::fence_after();
        for (int c = 0; c < nk; ++c, ++gchunk) {
          const int st = gchunk % stages;
          const uint32_t ph = (gchunk / stages) & 1;
          if (!wait(&full[st], ph)) break;
          tc::fence_after();
          const uint32_t sA = tc::smem_u32(tiles + (size_t)st * stage_bytes);
          const uint32_t sB = sA + TILE_BYTES;
#pragma unroll
          for (int kk = 0; kk < KCH / 16; ++kk) {
            tc::umma(tmem, tc::make_desc(sA + kk * 2 * M_LBO, M_LBO, M_SBO),
                     tc::make_desc(sB + kk * 2 * M_LBO, M_LBO, M_SBO), idesc,
                     (c > 0 || kk > 0) ? 1u : 0u);
          }
          tc::umma_commit(&empty[st]);
        }
        tc::umma_commit(tmem_full);
        ++proc;
      }
      // drain: every MMA issued by this thread has completed before TMEM is freed
      tc::umma_commit(drain);
      int zero = 0;
      tc::mbar_wait(drain, 0, &zero, &g_mlp_timeouts, MLP_TIMEOUT_NS);
    }
    __syncwarp();
  } else {
    // ======================== epilogue: warp w reads TMEM lanes 32w..32w+31 (tile rows)
    const int row = warp * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t proc = 0;
    for (long long w = blockIdx.x; w < items && !*abort_flag; w += gridDim.x) {
      const int m0 = (int)(w / nt) * 128, n0 = (int)(w % nt) * 128;
      if (!wait(tmem_full, proc & 1)) break;
      tc::fence_after();
      const int m = m0 + row;
      for (int j0 = 0; j0 < 128; j0 += 16) {
        uint32_t r[16];
        tc::tmem_ld16(lane_base + j0, r);
        tc::tmem_wait_ld();
        if (m < g.M) {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            const int n = n0 + j0 + jj;
            if (n >= g.N) continue;
            const float v = __uint_as_float(r[jj]);
            if (g.epi == EPI_BIAS_GELU) {
              const float x = v + g.bias[n];
              g.pre[(long long)m * g.ldp + n] = x;
              g.act[(long long)m * g.lda + n] = f2bf(gelu(x));
            } else {
              float* cp = g.C + (long long)m * g.scm + (long long)n * g.scn;
              float o = v;
              if (g.epi == EPI_BIAS) o += g.bias[n];
              else if (g.beta != 0.0f) o += g.beta * *cp;
              *cp = o;
            }
          }
        }
      }
      tc::fence_before();
      tc::mbar_arrive(tmem_empty);
      ++proc;
    }
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == MLP_MMA_WARP) tc::tmem_dealloc(tmem, 128);
}

// dpre = dact * GELU'(pre)
__global__ void gelu_bwd_kernel(long long count, const float* dact, const float* pre, float* dpre) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    dpre[i] = dact[i] * gelu_grad(pre[i]);
}

// out[n] += sum_m X[m*N + n]   (block 32 x 8: columns x row phases; out zeroed by the caller)
__global__ void colsum_kernel(int M, int N, const float* X, float* out) {
  __shared__ float part[8][33];
  const int n = blockIdx.x * 32 + threadIdx.x;
  float s = 0.0f;
  if (n < N)
    for (int m = blockIdx.y * 8 + threadIdx.y; m < M; m += gridDim.y * 8)
      s += X[(long long)m * N + n];
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && n < N) {
    float t = 0.0f;
#pragma unroll
    for (int r = 0; r < 8; ++r) t += part[r][threadIdx.x];
    atomicAdd(&out[n], t);
  }
}

// loss += sum (y - t)^2 / count ; dy = 2 (y - t) / count
__global__ void mse_kernel(long long count, const float* y, const float* t, float* dy,
                           double* loss) {
  const float inv = 1.0f / (float)count;
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = 2.0f * d * inv;
    acc += (double)d * d;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / (double)count);
}

// AdamW (decoupled weight decay) on the FP32 master parameters, then the BF16 copy
__global__ void adamw_kernel(long long count, float* w, const float* grad, float* m, float* v,
                             float lr, float b1, float b2, float eps, float wd, float bc1,
                             float bc2, uint16_t* wb) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] * (1.0f - lr * wd);
    wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    wb[i] = f2bf(wi);
  }
}

__global__ void to_bf16_kernel(long long count, const float* w, uint16_t* wb) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    wb[i] = f2bf(w[i]);
}

inline unsigned grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (unsigned)std::max<long long>(1, std::min<long long>(g, 4096));
}

template <typename TA, typename TB>
cudaError_t gemm(const MlpGemm& g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  constexpr int stages = 4;
  const size_t smem = (size_t)stages * 2 * TILE_BYTES + 1024;
  cudaError_t e = cudaFuncSetAttribute(mlp_gemm_kernel<TA, TB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const long long items = (long long)((g.M + 127) / 128) * ((g.N + 127) / 128);
  const int grid = (int)std::min<long long>(items, sms);
  mlp_gemm_kernel<TA, TB><<<grid, MLP_THREADS, smem, s>>>(g, stages);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

int mlp_timeouts_and_reset() {
  int h = 0, z = 0;
  cudaMemcpyFromSymbol(&h, g_mlp_timeouts, sizeof(int));
  if (h) cudaMemcpyToSymbol(g_mlp_timeouts, &z, sizeof(int));
  return h;
}

}  // namespace qt

using qt::MlpGemm;

// ============================================================== the network object
struct qt_mlp {
  qt_ctx* ctx = nullptr;
  int device = 0;
  int n_in = 0, width = 0, depth = 0, n_out = 0, max_batch = 0;
  std::vector<int> din, dout;         // per linear layer
  std::vector<long long> woff, boff;  // offsets of W_l (dout x din, row-major) and b_l
  long long nparams = 0;
  int step = 0;
  void* mem = nullptr;  // one allocation holds everything below
  float *w = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  uint16_t* wb = nullptr;
  float* pre = nullptr;     // [depth][max_batch][width]
  uint16_t* act = nullptr;  // [depth][max_batch][width]
  float *dact = nullptr, *dpre = nullptr;  // [max_batch][width]
  float *y = nullptr, *dy = nullptr;       // [max_batch][n_out]
  float *xin = nullptr, *tin = nullptr;    // staging for host inputs
  double* loss = nullptr;
};

namespace {

constexpr float ADAM_B1 = 0.9f, ADAM_B2 = 0.999f, ADAM_EPS = 1e-8f;

uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <typename T>
T* carve(char*& p, size_t count) {
  T* r = reinterpret_cast<T*>(p);
  p += (count * sizeof(T) + 255) & ~size_t(255);
  return r;
}

qt_status gemm_call(cudaError_t e) {
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

// forward pass of `batch` rows of X (device, [batch][n_in]) into n->y
qt_status forward(qt_mlp* n, int batch, const float* X) {
  cudaStream_t s = qt::ctx_stream(n->ctx);
  const int L = n->depth + 1;
  const long long BW = (long long)n->max_batch * n->width;
  for (int l = 0; l < L; ++l) {
    MlpGemm g{};
    g.M = batch;
    g.N = n->dout[l];
    g.K = n->din[l];
    g.B = n->wb + n->woff[l];
    g.sbn = n->din[l];
    g.sbk = 1;
    g.A = l == 0 ? static_cast<const void*>(X) : static_cast<const void*>(n->act + (l - 1) * BW);
    g.sam = l == 0 ? n->n_in : n->width;
    g.sak = 1;
    g.bias = n->w + n->boff[l];
    if (l < L - 1) {
      g.epi = qt::EPI_BIAS_GELU;
      g.pre = n->pre + l * BW;
      g.ldp = n->width;
      g.act = n->act + l * BW;
      g.lda = n->width;
    } else {
      g.epi = qt::EPI_BIAS;
      g.C = n->y;
      g.scm = n->n_out;
      g.scn = 1;
    }
    QT_TRY(gemm_call(l == 0 ? qt::gemm<float, uint16_t>(g, s)
                            : qt::gemm<uint16_t, uint16_t>(g, s)));
  }
  return QT_OK;
}

// loss and gradients (n->grad, flat like the parameters) after forward() on the same X
qt_status backward(qt_mlp* n, int batch, const float* X, const float* T) {
  cudaStream_t s = qt::ctx_stream(n->ctx);
  const int L = n->depth + 1;
  const long long BW = (long long)n->max_batch * n->width;
  const long long cnt = (long long)batch * n->n_out;
  cudaMemsetAsync(n->loss, 0, sizeof(double), s);
  qt::mse_kernel<<<qt::grid_for(cnt), 256, 0, s>>>(cnt, n->y, T, n->dy, n->loss);
  qt::count_launch();
  for (int l = L - 1; l >= 0; --l) {
    const int in = n->din[l], out = n->dout[l];
    const float* dP = l == L - 1 ? n->dy : n->dpre;
    // dW_l[o][i] = sum_m dP[m][o] In[m][i]
    MlpGemm g{};
    g.M = out;
    g.N = in;
    g.K = batch;
    g.A = dP;
    g.sam = 1;
    g.sak = out;
    g.B = l == 0 ? static_cast<const void*>(X) : static_cast<const void*>(n->act + (l - 1) * BW);
    g.sbn = 1;
    g.sbk = l == 0 ? n->n_in : n->width;
    g.epi = qt::EPI_STORE;
    g.C = n->grad + n->woff[l];
    g.scm = in;
    g.scn = 1;
    QT_TRY(gemm_call(l == 0 ? qt::gemm<float, float>(g, s) : qt::gemm<float, uint16_t>(g, s)));
    // db_l[o] = sum_m dP[m][o]
    cudaMemsetAsync(n->grad + n->boff[l], 0, (size_t)out * sizeof(float), s);
    const dim3 cg((out + 31) / 32, std::min(64, (batch + 7) / 8));
    qt::colsum_kernel<<<cg, dim3(32, 8), 0, s>>>(batch, out, dP, n->grad + n->boff[l]);
    qt::count_launch();
    if (l > 0) {
      // dAct_{l-1}[m][i] = sum_o dP[m][o] W_l[o][i] ;  dPre_{l-1} = dAct * GELU'(pre)
      MlpGemm h{};
      h.M = batch;
      h.N = in;
      h.K = out;
      h.A = dP;
      h.sam = out;
      h.sak = 1;
      h.B = n->wb + n->woff[l];
      h.sbn = 1;
      h.sbk = in;
      h.epi = qt::EPI_STORE;
      h.C = n->dact;
      h.scm = in;
      h.scn = 1;
      QT_TRY(gemm_call(qt::gemm<float, uint16_t>(h, s)));
      const long long c2 = (long long)batch * in;
      qt::gelu_bwd_kernel<<<qt::grid_for(c2), 256, 0, s>>>(c2, n->dact, n->pre + (l - 1) * BW,
                                                            n->dpre);
      qt::count_launch();
    }
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

qt_status sync_and_check(qt_mlp* n) {
  cudaStream_t s = qt::ctx_stream(n->ctx);
  QT_CUDA_TRY(cudaStreamSynchronize(s));
  if (qt::mlp_timeouts_and_reset()) QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  return QT_OK;
}

// device copies of the inputs (staged when they are host pointers)
qt_status inputs(qt_mlp* n, int batch, const float* X, const float* T, unsigned flags,
                 const float** Xd, const float** Td) {
  if (!n || !X || batch <= 0 || batch > n->max_batch) QT_FAIL(QT_ERR_ARG, "bad batch or input");
  cudaSetDevice(n->device);
  cudaStream_t s = qt::ctx_stream(n->ctx);
  if (flags & QT_FLAG_DEVICE_POINTERS) {
    *Xd = X;
    if (Td) *Td = T;
    return QT_OK;
  }
  cudaMemcpyAsync(n->xin, X, (size_t)batch * n->n_in * sizeof(float), cudaMemcpyHostToDevice, s);
  *Xd = n->xin;
  if (Td && T) {
    cudaMemcpyAsync(n->tin, T, (size_t)batch * n->n_out * sizeof(float), cudaMemcpyHostToDevice,
                    s);
    *Td = n->tin;
  }
  return QT_OK;
}

}  // namespace

extern "C" qt_status qt_mlp_create(qt_ctx* ctx, int n_in, int width, int depth, int n_out,
                                   int max_batch, const float* init_params, uint64_t seed,
                                   qt_mlp** out) {
  if (!ctx || !out || n_in <= 0 || width <= 0 || depth <= 0 || n_out <= 0 || max_batch <= 0)
    QT_FAIL(QT_ERR_ARG, "bad network dimensions");
  qt_mlp* n = new qt_mlp();
  n->ctx = ctx;
  n->device = qt::ctx_device(ctx);
  n->n_in = n_in; n->width = width; n->depth = depth; n->n_out = n_out;
  n->max_batch = max_batch;
  for (int l = 0; l <= depth; ++l) {
    const int din = l == 0 ? n_in : width, dout = l == depth ? n_out : width;
    n->din.push_back(din);
    n->dout.push_back(dout);
    n->woff.push_back(n->nparams);
    n->nparams += (long long)din * dout;
    n->boff.push_back(n->nparams);
    n->nparams += dout;
  }
  const size_t P = (size_t)n->nparams, MB = (size_t)max_batch;
  size_t bytes = 0;
  auto add = [&](size_t b) { bytes += (b + 255) & ~size_t(255); };
  add(P * 4); add(P * 4); add(P * 4); add(P * 4); add(P * 2);
  add(depth * MB * width * 4); add(depth * MB * width * 2);
  add(MB * width * 4); add(MB * width * 4);
  add(MB * n_out * 4); add(MB * n_out * 4);
  add(MB * n_in * 4); add(MB * n_out * 4); add(8);
  cudaSetDevice(n->device);
  if (cudaMalloc(&n->mem, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete n;
    QT_FAIL(QT_ERR_NOMEM, "network allocation failed");
  }
  char* p = reinterpret_cast<char*>(n->mem);
  n->w = carve<float>(p, P); n->grad = carve<float>(p, P);
  n->m = carve<float>(p, P); n->v = carve<float>(p, P);
  n->wb = carve<uint16_t>(p, P);
  n->pre = carve<float>(p, depth * MB * width);
  n->act = carve<uint16_t>(p, depth * MB * width);
  n->dact = carve<float>(p, MB * width); n->dpre = carve<float>(p, MB * width);
  n->y = carve<float>(p, MB * n_out); n->dy = carve<float>(p, MB * n_out);
  n->xin = carve<float>(p, MB * n_in); n->tin = carve<float>(p, MB * n_out);
  n->loss = carve<double>(p, 1);
  // Glorot-uniform weights, zero biases (or the caller's parameters)
  std::vector<float> h(P, 0.0f);
  if (init_params) {
    std::memcpy(h.data(), init_params, P * sizeof(float));
  } else {
    uint64_t st = seed;
    for (int l = 0; l <= depth; ++l) {
      const double a = std::sqrt(6.0 / (double)(n->din[l] + n->dout[l]));
      for (long long i = 0; i < (long long)n->din[l] * n->dout[l]; ++i) {
        const double u = (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
        h[n->woff[l] + i] = (float)((2.0 * u - 1.0) * a);
      }
    }
  }
  cudaStream_t s = qt::ctx_stream(ctx);
  cudaMemcpyAsync(n->w, h.data(), P * sizeof(float), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(n->m, 0, P * sizeof(float), s);
  cudaMemsetAsync(n->v, 0, P * sizeof(float), s);
  qt::to_bf16_kernel<<<qt::grid_for((long long)P), 256, 0, s>>>((long long)P, n->w, n->wb);
  qt::count_launch();
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    const char* msg = cudaGetErrorString(cudaGetLastError());
    cudaFree(n->mem);
    delete n;
    QT_FAIL(QT_ERR_CUDA, msg);
  }
  *out = n;
  return QT_OK;
}

extern "C" qt_status qt_mlp_destroy(qt_mlp* n) {
  if (!n) return QT_OK;
  cudaSetDevice(n->device);
  cudaStream_t s = qt::ctx_stream(n->ctx);
  cudaStreamSynchronize(s);
  cudaFree(n->mem);
  delete n;
  return QT_OK;
}

extern "C" qt_status qt_mlp_num_params(const qt_mlp* n, int64_t* count) {
  if (!n || !count) QT_FAIL(QT_ERR_ARG, "null argument");
  *count = n->nparams;
  return QT_OK;
}

extern "C" qt_status qt_mlp_get_params(qt_mlp* n, float* host) {
  if (!n || !host) QT_FAIL(QT_ERR_ARG, "null argument");
  cudaSetDevice(n->device);
  cudaStream_t s = qt::ctx_stream(n->ctx);
  cudaMemcpyAsync(host, n->w, (size_t)n->nparams * sizeof(float), cudaMemcpyDeviceToHost, s);
  return sync_and_check(n);
}

extern "C" qt_status qt_mlp_set_params(qt_mlp* n, const float* host) {
  if (!n || !host) QT_FAIL(QT_ERR_ARG, "null argument");
  cudaSetDevice(n->device);
  cudaStream_t s = qt::ctx_stream(n->ctx);
  const long long P = n->nparams;
  cudaMemcpyAsync(n->w, host, (size_t)P * sizeof(float), cudaMemcpyHostToDevice, s);
  qt::to_bf16_kernel<<<qt::grid_for(P), 256, 0, s>>>(P, n->w, n->wb);
  qt::count_launch();
  return sync_and_check(n);
}

extern "C" qt_status qt_mlp_infer(qt_mlp* n, int batch, const float* X, float* Y, unsigned flags) {
  const float* Xd = nullptr;
  QT_TRY(inputs(n, batch, X, nullptr, flags, &Xd, nullptr));
  if (!Y) QT_FAIL(QT_ERR_ARG, "null output");
  QT_TRY(forward(n, batch, Xd));
  cudaStream_t s = qt::ctx_stream(n->ctx);
  const size_t yb = (size_t)batch * n->n_out * sizeof(float);
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  cudaMemcpyAsync(Y, n->y, yb, devp ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s);
  if (!devp || (flags & QT_FLAG_SYNC)) return sync_and_check(n);
  return QT_OK;
}

extern "C" qt_status qt_mlp_grad(qt_mlp* n, int batch, const float* X, const float* T,
                                 float* grad_host, double* loss, unsigned flags) {
  const float *Xd = nullptr, *Td = nullptr;
  if (!T || !grad_host) QT_FAIL(QT_ERR_ARG, "null argument");
  QT_TRY(inputs(n, batch, X, T, flags, &Xd, &Td));
  QT_TRY(forward(n, batch, Xd));
  QT_TRY(backward(n, batch, Xd, Td));
  cudaStream_t s = qt::ctx_stream(n->ctx);
  cudaMemcpyAsync(grad_host, n->grad, (size_t)n->nparams * sizeof(float), cudaMemcpyDeviceToHost,
                  s);
  if (loss) cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
  return sync_and_check(n);
}

extern "C" qt_status qt_mlp_train_step(qt_mlp* n, int batch, const float* X, const float* T,
                                       float lr, float weight_decay, double* loss,
                                       unsigned flags) {
  const float *Xd = nullptr, *Td = nullptr;
  if (!T) QT_FAIL(QT_ERR_ARG, "null target");
  QT_TRY(inputs(n, batch, X, T, flags, &Xd, &Td));
  QT_TRY(forward(n, batch, Xd));
  QT_TRY(backward(n, batch, Xd, Td));
  ++n->step;
  const float bc1 = 1.0f - (float)std::pow((double)ADAM_B1, n->step);
  const float bc2 = 1.0f - (float)std::pow((double)ADAM_B2, n->step);
  const long long P = n->nparams;
  cudaStream_t s = qt::ctx_stream(n->ctx);
  qt::adamw_kernel<<<qt::grid_for(P), 256, 0, s>>>(P, n->w, n->grad, n->m, n->v, lr, ADAM_B1,
                                                   ADAM_B2, ADAM_EPS, weight_decay, bc1, bc2,
                                                   n->wb);
  qt::count_launch();
  if (loss) {
    cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
    return sync_and_check(n);
  }
  if (flags & QT_FLAG_SYNC) return sync_and_check(n);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}
