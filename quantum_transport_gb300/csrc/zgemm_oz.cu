// Split-precision complex block product on the 5th-generation tensor cores
// (tcgen05.mma kind::f16, BF16 x BF16 -> FP32 in TMEM), Ozaki-style.
//
//   C_b = alpha * op(A_b) op(B_b) + beta * D_b + z_b I     (n <= 128, real alpha/beta)
//
// This is the GB300 replacement of the reference's per-slab zgemm calls
// (src/cuda_rgf_mod.f90:152-175, 293-370; Sancho :698-712) for the
// split-precision path.  GB300's FP64 pipes run at ~1 TFLOP/s, so FP64-grade
// products are rebuilt from exact BF16 digit products:
//
//  * complex -> real: with At = op(A), Bt = op(B) (n x n complex), the real K
//    axis interleaves the real and imaginary parts of each complex k:
//      A' row i = (Re At[i,k], Im At[i,k])_k
//      Cr: B' column j = (Re Bt[k,j], -Im Bt[k,j])_k    Ci: (Im Bt[k,j], Re Bt[k,j])_k
//    so each complex element is loaded once per stage.  One CTA work item is one
//    real part of one NT-column tile (M = 128 padded rows, K' = 2n).  For
//    complex64 operands one item computes both parts: Ci = A'' B'_r with
//    A'' row i = (Im At[i,k], -Re At[i,k])_k written from the same digits as A',
//    so each operand is split once per item;
//  * digits: every row i of A' is scaled by 2^-e_i (e_i: exponent bound of the
//    row's largest entry, |entry| < 2^(e_i-1), from the prologue kernel) and
//    written as S balanced base-256 digits D_s = d_s 2^(-8s), |d_s| <= 128 --
//    each exactly representable in BF16.  Columns of B' likewise with f_j;
//  * products: all digit pairs (s, t) with s + t <= L are issued; pair level
//    l = s + t accumulates into TMEM accumulator min(l, NACC - 1), where the 512
//    TMEM columns hold NACC = 512 / (NT x parts) accumulators (8 for the
//    complex128 products with NT = 64; 2 per part for complex64 with both
//    parts, levels 1-3 sharing the second).  A level-l partial sum is an integer
//    multiple of 2^(-8l) below (l+1) 2^14 K' 2^(-8l), so levels l <= 3 are EXACT
//    in FP32 for K' <= 256; a higher level on its own accumulator rounds at
//    2^(-24-8l) <= 2^-56 of the row/column scale, and the shared complex64
//    accumulator rounds at about 2^-32 per MMA, ~2^-28 of the result;
//  * epilogue: the accumulators are summed in double-float FP32 arithmetic
//    (TwoSum), scaled by 2^(e_i + f_j - 16), and written as FP32 (complex64
//    output) or assembled into FP64 bits with integer operations (complex128
//    output, no use of the FP64 pipe).
//
// Two kernel families share the digit arithmetic below: the register-staged kernel
// (zgemm_oz_kernel, producers slice digits straight from global loads) and the TMA-fed
// kernels further down (zgemm_c64_tma_kernel, zgemm_c128_tma_kernel: raw tiles copied
// into shared memory by cp.async.bulk.tensor, digits sliced shared memory to shared
// memory), which run whenever both operands can be addressed by a tensor map.
//
// Roles of the register-staged kernel (one CTA per SM: the accumulators use all 512 TMEM
// columns): warps 0-3
// epilogue (TMEM lanes 0-127); 16 producer warps for 128-column tiles, 8 for
// 64-column tiles (digit slicing straight from global memory into the
// canonical no-swizzle K-major UMMA layout in shared memory); the last warp
// allocates TMEM and holds the single MMA-issuing thread.  Stages are handed over with mbarriers; every wait is
// bounded (a few seconds) and records a timeout instead of hanging.
#include <cuda.h>
#include <stdint.h>

#include "qt_common.cuh"
#include "qt_kernels.h"
#include "tc_ptx.cuh"

namespace qt {

__device__ int g_oz_timeouts = 0;

namespace {

constexpr int KC = 32;            // real-K elements per pipeline stage
// Roles per CTA: warps 0-3 epilogue, then the producer warps, then the MMA warp.
// 128-column tiles get 16 producer warps (more loads in flight per SM), 64-column
// tiles 8, so that each producer thread stages a whole number of items.
template <int NT>
struct Roles {
  static constexpr int NPROD = NT == 128 ? 512 : 256;
  static constexpr int NTHREADS = 128 + NPROD + 32;
  static constexpr int MMA_WARP = 4 + NPROD / 32;
};
constexpr uint64_t TIMEOUT_NS = 4000000000ull;  // 4 s per wait
constexpr int PLANE_BYTES = 128 * KC * 2;       // one digit plane of a 128-row tile: 8 KB
constexpr uint32_t LBO = 128;                   // K-adjacent core matrices
constexpr uint32_t SBO = (KC / 8) * 128;        // 8-row groups

using tc::fence_proxy_async;
using tc::make_idesc;
using tc::mbar_arrive;
using tc::mbar_init;
using tc::smem_u32;
using tc::tmem_ld16;
using tc::tmem_ld8;
using tc::tmem_wait_ld;
using tc::umma;
using tc::umma_commit;

// bounded wait (4 s); a timeout raises the CTA's abort flag and counts in *tcount
// (GemmArgs::timeouts, else g_oz_timeouts)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* tcount) {
  return tc::mbar_wait(bar, parity, abort_flag, tcount, TIMEOUT_NS);
}
__device__ __forceinline__ void tc_fence_before() { tc::fence_before(); }
__device__ __forceinline__ void tc_fence_after() { tc::fence_after(); }
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) { return tc::make_desc(saddr, LBO, SBO); }

// ------------------------------------------------------------ element access
template <typename T> struct Elem;
template <> struct Elem<float2> {
  __device__ static float2 ld(const void* p, long long off) {
    return reinterpret_cast<const float2*>(p)[off];
  }
};
template <> struct Elem<double2> {
  __device__ static double2 ld(const void* p, long long off) {
    return reinterpret_cast<const double2*>(p)[off];
  }
};

// element (r, c) of op(M); part 0 = real, 1 = imaginary (conjugated for OP_C)
template <typename T>
__device__ __forceinline__ T load_op(const void* M, int ld, int op, int r, int c) {
  if (op == OP_N) return Elem<T>::ld(M, r + (long long)c * ld);
  T v = Elem<T>::ld(M, c + (long long)r * ld);
  if (op == OP_C) v.y = -v.y;
  return v;
}

// |x| as ordered integer bits (non-negative floats compare like their bit patterns)
__device__ __forceinline__ unsigned long long absbits(double2 v, int part) {
  return (unsigned long long)__double_as_longlong(part ? v.y : v.x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long absbits(float2 v, int part) {
  return __float_as_uint(part ? v.y : v.x) & 0x7FFFFFFFu;
}
// exponent bound e with max|x| < 2^(e-1) from the bits of max|x|; 0 for a zero vector
template <typename T> __device__ __forceinline__ int exp_bound_bits(unsigned long long mb);
template <> __device__ __forceinline__ int exp_bound_bits<double2>(unsigned long long mb) {
  const int ef = (int)((mb >> 52) & 0x7FF);
  return ef ? ef - 1023 + 2 : 0;
}
template <> __device__ __forceinline__ int exp_bound_bits<float2>(unsigned long long mb) {
  const int ef = (int)((mb >> 23) & 0xFF);
  return ef ? ef - 127 + 2 : 0;
}

// ------------------------------------------------------------ digit slicing
// FP32 value: y = x 2^(8-e) in (-128, 128); digits D_s = d_s 2^-8s by magic rounding
template <int S>
__device__ __forceinline__ void digits_f32(float x, float scale, float* D) {
  float r = x * scale;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const float M = 12582912.0f * __int_as_float((127 - 8 * s) << 23);  // 1.5 * 2^(23 - 8s)
    const float d = (r + M) - M;
    D[s] = d;
    r -= d;
  }
}
// The same digits for a (Re, Im) pair with the packed FP32x2 arithmetic of sm_100+
// (each lane rounded exactly as the scalar form: bit-identical digits).
template <int S>
__device__ __forceinline__ void digits_f32x2(float2 x, float scale, float2* D) {
  float2 r = __fmul2_rn(x, make_float2(scale, scale));
  const float2 mone = make_float2(-1.0f, -1.0f);
#pragma unroll
  for (int s = 0; s < S; ++s) {
    const float M = 12582912.0f * __int_as_float((127 - 8 * s) << 23);  // 1.5 * 2^(23 - 8s)
    const float2 d = __fadd2_rn(__fadd2_rn(r, make_float2(M, M)), make_float2(-M, -M));
    D[s] = d;
    r = __ffma2_rn(d, mone, r);  // r - d, exact
  }
}
// the BF16 halves (upper 16 bits) of lo and hi in one 32-bit word: digits carry <= 8
// significant bits, so the truncation is exact
__device__ __forceinline__ uint32_t pack_pair(float2 d) {
  return __byte_perm(__float_as_uint(d.x), __float_as_uint(d.y), 0x7632);
}
// FP64 value via integer arithmetic on its bits: T = round(x 2^(8S - e)), balanced digits
template <int S>
__device__ __forceinline__ void digits_f64(double x, int e, float* D) {
  const long long bits = __double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  long long T = 0;
  if (ex != 0) {
    const long long m = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
    const int sh = ex - 1075 + 8 * S - e;
    if (sh >= 0) T = m << sh;
    else if (sh > -63) T = (m + (1ll << (-sh - 1))) >> (-sh);
    if (bits < 0) T = -T;
  }
  // Balanced digits d_s in [-128, 127], T = sum_s d_s 256^(S-1-s), without the digit-by-digit
  // carry loop: with V = T + 128 (1 + 256 + ... + 256^(S-2)), byte j of V is d_(S-1-j) + 128
  // for j < S-1 (each byte's +128 absorbs the borrow of the digit below it), and
  // V >> 8(S-1) is d_0.
  unsigned long long K = 0;
#pragma unroll
  for (int j = 0; j < S - 1; ++j) K |= 0x80ull << (8 * j);
  const unsigned long long V = (unsigned long long)T + K;
#pragma unroll
  for (int j = 0; j < S - 1; ++j) {
    const int s = S - 1 - j;
    const unsigned byte = (unsigned)(V >> (8 * j)) & 255u;
    const float sc = __int_as_float((127 - 8 * s) << 23);  // 2^-8s
    // (12582912 + byte) 2^-8s - 12583040 2^-8s = (byte - 128) 2^-8s, exact in one FMA
    D[s] = fmaf(__uint_as_float(0x4B400000u | byte), sc, -12583040.0f * sc);
  }
  const int top = (int)((long long)V >> (8 * (S - 1)));
  D[0] = __int_as_float(0x4B400000 + top) - 12582912.0f;  // exact float(d_0)
}
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  // the digits carry <= 8 significant bits: truncation to BF16 is exact
  return (__float_as_uint(lo) >> 16) | (__float_as_uint(hi) & 0xFFFF0000u);
}

// ------------------------------------------------------------ epilogue math
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// (hi + lo) * 2^e2 -> FP64 bits with integer operations; |lo| <= ulp(hi)/2
__device__ __forceinline__ double df_to_double(float hi, float lo, int e2) {
  const uint32_t hb = __float_as_uint(hi);
  if ((hb & 0x7FFFFFFFu) == 0) return 0.0;
  const uint32_t sgn = hb >> 31;
  int eh = (int)((hb >> 23) & 0xFF);
  unsigned long long M;
  if (eh == 0) {  // subnormal hi: value tiny, keep what is there
    M = (unsigned long long)(hb & 0x7FFFFF) << 29;
    eh = 1;
    while (M && !(M >> 52)) { M <<= 1; --eh; }
  } else {
    M = (unsigned long long)((hb & 0x7FFFFF) | 0x800000) << 29;
  }
  const uint32_t lb = __float_as_uint(lo);
  if ((lb & 0x7FFFFFFFu) != 0) {
    int el = (int)((lb >> 23) & 0xFF);
    unsigned long long ml = (lb & 0x7FFFFF) | (el ? 0x800000u : 0u);
    if (!el) el = 1;
    const int s = 29 - (eh - el);
    unsigned long long L = 0;
    if (s >= 0) L = ml << s;
    else if (s > -63) L = (ml + (1ull << (-s - 1))) >> (-s);
    if ((lb >> 31) == sgn) M += L; else M -= L;
    if (M >> 53) { M = (M + 1) >> 1; ++eh; }
    while (M && !(M >> 52)) { M <<= 1; --eh; }
  }
  const int E = eh - 127 + 1023 + e2;
  if (E <= 0 || M == 0) return sgn ? -0.0 : 0.0;
  if (E >= 2047) return __longlong_as_double(((long long)sgn << 63) | 0x7FF0000000000000ll);
  const unsigned long long out = ((unsigned long long)sgn << 63) | ((unsigned long long)E << 52) |
                                 (M & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)out);
}

template <typename T> struct Store;
template <> struct Store<float2> {
  // acc -> value (already combined as hi/lo), adds beta*D and z on the diagonal
  __device__ static void put(void* C, long long off, int part, float hi, float lo, int e2,
                             float alpha, float beta, const void* D, long long doff, bool diag,
                             double zpart) {
    float v, w;
    if (e2 > -126 && e2 < 128) {
      const float sc = __int_as_float((127 + e2) << 23);  // 2^e2
      v = alpha * (hi * sc);
      w = alpha * (lo * sc);
    } else {
      v = alpha * ldexpf(hi, e2);
      w = alpha * ldexpf(lo, e2);
    }
    if (D) v = fmaf(beta, reinterpret_cast<const float*>(D)[2 * doff + part], v);
    if (diag) v += (float)zpart;
    reinterpret_cast<float*>(C)[2 * off + part] = v + w;
  }
};
template <> struct Store<double2> {
  __device__ static void put(void* C, long long off, int part, float hi, float lo, int e2,
                             float alpha, float beta, const void* D, long long doff, bool diag,
                             double zpart) {
    double v = df_to_double(alpha * hi, alpha * lo, e2);
    if (D) v = fma((double)beta, reinterpret_cast<const double*>(D)[2 * doff + part], v);
    if (diag) v += zpart;
    reinterpret_cast<double*>(C)[2 * off + part] = v;
  }
};

// ------------------------------------------------------------ scale prologue
// scales[b][0..127]   = e_i: exponent bound of row i of op(A)   over Re and Im parts
// scales[b][128..255] = f_j: exponent bound of column j of op(B)
// One CTA per (batch entry, operand).  A vector is either contiguous in memory
// (warp per vector, lanes along it) or strided (threads along consecutive
// vectors, which coalesces the loads across the warp); loads are unrolled so
// many are in flight.
template <typename TIn>
__global__ void __launch_bounds__(256) oz_scales_kernel(GemmArgs a) {
  __shared__ unsigned long long part_max[256];
  const int which = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nv = which ? a.n : a.m, K = a.k;  // vectors (rows of op(A) / columns of op(B)), length
  for (long long b = blockIdx.x; b < a.batch; b += gridDim.x) {
    int* out = a.scales + b * 256 + which * 128;
    if (a.active && !a.active[b]) continue;
    const int op = which ? a.opB : a.opA;
    const BatchRef& R = which ? a.B : a.A;
    const TIn* M = batch_ptr<const TIn>(R, b);
    const int ld = R.ld;
    // row of op(A) = storage row (OP_N) / storage column (else); column of op(B) = storage
    // column (OP_N) / storage row (else)
    const bool contiguous = which ? (op == OP_N) : (op != OP_N);
    if (contiguous) {
      for (int v = warp; v < 128; v += 8) {
        unsigned long long m = 0;
        if (v < nv) {
#pragma unroll 4
          for (int e = lane; e < K; e += 32) {
            const TIn x = M[e + (long long)v * ld];
            m = max(m, max(absbits(x, 0), absbits(x, 1)));
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) out[v] = v < nv ? exp_bound_bits<TIn>(m) : 0;
      }
    } else {
      const int v = tid & 127, h = tid >> 7;  // two threads per vector
      unsigned long long m = 0;
      if (v < nv) {
#pragma unroll 8
        for (int e = h; e < K; e += 2) {
          const TIn x = M[v + (long long)e * ld];
          m = max(m, max(absbits(x, 0), absbits(x, 1)));
        }
      }
      part_max[tid] = m;
      __syncthreads();
      if (h == 0) out[v] = v < nv ? exp_bound_bits<TIn>(max(m, part_max[tid + 128])) : 0;
      __syncthreads();
    }
  }
}

// ------------------------------------------------------------ the kernel
template <int S, int L, int NT, typename TIn, typename TOut>
__global__ void __launch_bounds__(Roles<NT>::NTHREADS, 1) zgemm_oz_kernel(GemmArgs a, int stages) {
  constexpr int NPROD = Roles<NT>::NPROD, MMA_WARP = Roles<NT>::MMA_WARP;
  // Complex64 operands: one work item computes both real parts of C.  The imaginary
  // part uses the real part's B' planes against a second A layout A'' = (Im A, -Re A),
  // written from the same digits (negating a balanced digit is exact), so A and B are
  // split once per item, not once per part.
  constexpr bool BOTH = sizeof(TIn) == 8;
  constexpr int NPARTS = BOTH ? 2 : 1;
  // NT output columns per CTA; the 512 TMEM columns hold 512/NT accumulators, shared by
  // the parts of an item.  With NT = 64 and one part every digit level up to 7 has its
  // own (exact) accumulator; complex64 with both parts keeps level 0 exact and sums
  // levels 1-3 in one FP32 accumulator (about 2^-28 of the result, below its 2^-24).
  constexpr int NACC_MAX = 512 / (NT * NPARTS);
  constexpr int NACC = (L + 1 < NACC_MAX) ? L + 1 : NACC_MAX;
  constexpr int BPLANE = NT * KC * 2;  // one B digit plane of an NT-row tile
  constexpr int APLANES = NPARTS;      // A digit layouts per stage
  constexpr int ITEMS = (512 + 4 * NT) / NPROD;  // (row, 8-K group) items per producer thread
  static_assert((512 + 4 * NT) % NPROD == 0, "item split");
  extern __shared__ __align__(1024) unsigned char smem[];
  // carve: [stages x (A planes | B planes)] [barriers] [tmem slot, abort flag]
  const int stage_bytes = S * (APLANES * PLANE_BYTES + BPLANE);
  unsigned char* tiles = smem;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)stages * stage_bytes);
  uint64_t* full = bars;                 // [stages] producers -> MMA
  uint64_t* empty = bars + stages;       // [stages] MMA (commit) -> producers
  uint64_t* tmem_full = bars + 2 * stages;  // MMA (commit) -> epilogue
  uint64_t* tmem_empty = tmem_full + 1;     // epilogue -> MMA
  uint64_t* drain = tmem_full + 2;          // teardown
  uint32_t* tmem_base_sm = reinterpret_cast<uint32_t*>(tmem_full + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_base_sm + 1);
  int* const tcount = a.timeouts ? a.timeouts : &g_oz_timeouts;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = a.m, n = a.n, K = a.k;         // C is m x n, op(A) m x K, op(B) K x n
  const int npad = (n + 15) & ~15;
  const int nch = (K + KC / 2 - 1) / (KC / 2);  // stages: KC real K = KC/2 complex k each
  const int ntile = (npad + NT - 1) / NT;  // column tiles per real part
  // work item: (batch entry, real/imag part of C unless BOTH, column tile)
  const long long nitems = (BOTH ? 1LL : 2LL) * ntile * a.batch;

  if (tid == 0) {
    for (int s = 0; s < stages; ++s) { mbar_init(&full[s], NPROD); mbar_init(&empty[s], 1); }
    mbar_init(tmem_full, 1);
    mbar_init(tmem_empty, 128);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP) {
    tc::tmem_alloc(tmem_base_sm, 512);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_base_sm;

  if (warp >= 4 && warp < MMA_WARP) {
    // ======================== producers
    const int p = tid - 128;  // 0 .. NPROD-1
    uint32_t proc = 0, gchunk = 0;
    if constexpr (BOTH) {
      // Complex64: thread p stages row r of op(A) and column ct*NT + r of op(B), both in
      // 8-K group g of every stage.  Pointers, k strides, signs and scales are fixed per
      // work item.  Where an operand's k run is contiguous (op(A) transposed, op(B) = N)
      // and 16-byte aligned, its four complex k of a stage come in two 16-byte loads.
      static_assert(NPROD == 512 && NT == 128 && ITEMS == 2, "complex64 producer layout");
      const int r = p & 127, g = p >> 7;
      const uint32_t off = (uint32_t)((r >> 3) * SBO + g * LBO + (r & 7) * 16);
      for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
        const long long b = w / ntile;
        const int ct = (int)(w % ntile);
        if (a.active && !a.active[b]) continue;
        const TIn* A = batch_ptr<const TIn>(a.A, b);
        const TIn* B = batch_ptr<const TIn>(a.B, b);
        const int* erow = a.scales + b * 256;
        const int* fcol = erow + 128;
        const int rb = ct * NT + r;  // column of op(B)
        const bool okA = r < m, okB = rb < n;
        const long long ldA = a.A.ld, ldB = a.B.ld;
        const long long offA = a.opA == OP_N ? r : (long long)r * ldA;
        const long long ksA = a.opA == OP_N ? ldA : 1;
        const long long offB = a.opB == OP_N ? (long long)rb * ldB : rb;
        const long long ksB = a.opB == OP_N ? 1 : ldB;
        // k0 below is even, so element offset offX + k0 is even when ldX is
        const bool vecA = ksA == 1 && (ldA & 1) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
        const bool vecB = ksB == 1 && (ldB & 1) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
        // A' = (Re, Im) of op(A); B' real layout = (Re, -Im) of op(B); OP_C conjugates
        const float sA = a.opA == OP_C ? -1.f : 1.f, sB = a.opB == OP_C ? 1.f : -1.f;
        // 2^(8-e) as pre * scale: rows below 2^-119 would overflow a single FP32 power of
        // two, so they are first lifted by 2^64 (exact).  Rows past m / n are zero.
        const int eA = okA ? erow[r] : 0, eB = okB ? fcol[rb] : 0;
        const bool tA = eA < -118, tB = eB < -118;
        const float preA = tA ? 18446744073709551616.0f : 1.0f;
        const float preB = tB ? 18446744073709551616.0f : 1.0f;
        const float2 mA = make_float2(preA, preA * sA), mB = make_float2(preB, preB * sB);
        const float scA = __int_as_float((127 + 8 - (tA ? eA + 64 : eA)) << 23);
        const float scB = __int_as_float((127 + 8 - (tB ? eB + 64 : eB)) << 23);
        for (int c = 0; c < nch; ++c, ++gchunk) {
          const int st = gchunk % stages;
          const uint32_t ph = (gchunk / stages) & 1;
          unsigned char* stA = tiles + (size_t)st * stage_bytes;
          unsigned char* stB = stA + APLANES * S * PLANE_BYTES;
          const int k0 = c * (KC / 2) + 4 * g;
          // the stage's global loads do not need its slot: they are in flight while the
          // slot is being released
          TIn xa[4], xb[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            xa[u] = make_float2(0.f, 0.f);
            xb[u] = make_float2(0.f, 0.f);
          }
          if (k0 + 3 < K) {
            if (okA) {
              if (vecA) {
                const float4 v0 = *reinterpret_cast<const float4*>(A + offA + k0);
                const float4 v1 = *reinterpret_cast<const float4*>(A + offA + k0 + 2);
                xa[0] = make_float2(v0.x, v0.y); xa[1] = make_float2(v0.z, v0.w);
                xa[2] = make_float2(v1.x, v1.y); xa[3] = make_float2(v1.z, v1.w);
              } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) xa[u] = A[offA + (k0 + u) * ksA];
              }
            }
            if (okB) {
              if (vecB) {
                const float4 v0 = *reinterpret_cast<const float4*>(B + offB + k0);
                const float4 v1 = *reinterpret_cast<const float4*>(B + offB + k0 + 2);
                xb[0] = make_float2(v0.x, v0.y); xb[1] = make_float2(v0.z, v0.w);
                xb[2] = make_float2(v1.x, v1.y); xb[3] = make_float2(v1.z, v1.w);
              } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) xb[u] = B[offB + (k0 + u) * ksB];
              }
            }
          } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              if (k0 + u < K) {
                if (okA) xa[u] = A[offA + (k0 + u) * ksA];
                if (okB) xb[u] = B[offB + (k0 + u) * ksB];
              }
            }
          }
          if (!mbar_wait(&empty[st], ph ^ 1, abort_flag, tcount)) break;
          uint32_t pk[S][4], pk2[S][4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            float2 D[S];
            digits_f32x2<S>(__fmul2_rn(xa[u], mA), scA, D);
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2) {
              pk[s2][u] = pack_pair(D[s2]);
              pk2[s2][u] = pack_pair(make_float2(D[s2].y, D[s2].x)) ^ 0x80000000u;
            }
          }
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2) {
            *reinterpret_cast<uint4*>(stA + (size_t)s2 * PLANE_BYTES + off) =
                make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
            *reinterpret_cast<uint4*>(stA + (size_t)(S + s2) * PLANE_BYTES + off) =
                make_uint4(pk2[s2][0], pk2[s2][1], pk2[s2][2], pk2[s2][3]);
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            float2 D[S];
            digits_f32x2<S>(__fmul2_rn(xb[u], mB), scB, D);
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2) pk[s2][u] = pack_pair(D[s2]);
          }
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2)
            *reinterpret_cast<uint4*>(stB + (size_t)s2 * BPLANE + off) =
                make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
          fence_proxy_async();
          mbar_arrive(&full[st]);
        }
        ++proc;
      }
    } else
    for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
      const long long b = w / (NPARTS == 2 ? ntile : 2 * ntile);
      const int part = BOTH ? 0 : (int)((w / ntile) & 1), ct = (int)(w % ntile);
      if (a.active && !a.active[b]) continue;
      // batch strides are in complex elements: address through the element type
      const void* A = batch_ptr<const TIn>(a.A, b);
      const void* B = batch_ptr<const TIn>(a.B, b);
      const int* erow = a.scales + b * 256;  // row exponents of op(A) (prologue kernel)
      const int* fcol = erow + 128;          // column exponents of op(B)
      // ---- pipeline stages.  The real K axis interleaves (Re, Im) of each complex k:
      //   A' row i:      Re At[i,k], Im At[i,k]
      //   B' (C real):   Re Bt[k,j], -Im Bt[k,j]      B' (C imag): Im Bt[k,j], Re Bt[k,j]
      // so every complex element is loaded once; all loads of a stage are issued
      // before any digit arithmetic (memory-level parallelism).
      for (int c = 0; c < nch; ++c, ++gchunk) {
        const int st = gchunk % stages;
        const uint32_t ph = (gchunk / stages) & 1;
        unsigned char* stA = tiles + (size_t)st * stage_bytes;
        unsigned char* stB = stA + APLANES * S * PLANE_BYTES;
        const int kc0 = c * (KC / 2);  // complex k offset of this stage
        // loads first: they are in flight while the stage's slot is being released
        TIn xv[ITEMS][4];
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
          const int item = p + q * NPROD;
          const bool isA = item < 512;
          const int it2 = isA ? item : item - 512;
          const int r = isA ? (it2 & 127) : (it2 % NT), g = isA ? (it2 >> 7) : (it2 / NT);
          const int rg = isA ? r : ct * NT + r;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int k = kc0 + 4 * g + u;
            TIn x;
            x.x = 0; x.y = 0;
            if (rg < (isA ? m : n) && k < K)
              x = isA ? load_op<TIn>(A, a.A.ld, a.opA, rg, k) : load_op<TIn>(B, a.B.ld, a.opB, k, rg);
            xv[q][u] = x;
          }
        }
        if (!mbar_wait(&empty[st], ph ^ 1, abort_flag, tcount)) break;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
          const int item = p + q * NPROD;
          const bool isA = item < 512;
          const int it2 = isA ? item : item - 512;
          const int r = isA ? (it2 & 127) : (it2 % NT), g = isA ? (it2 >> 7) : (it2 / NT);
          const int rg = isA ? r : ct * NT + r;  // row of op(A) / column of op(B)
          const int e = isA ? erow[r] : (rg < n ? fcol[rg] : 0);
          uint32_t packed[S][4];
          uint32_t packed2[BOTH ? S : 1][4];  // A'' = (Im, -Re) of A items (BOTH)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            float D0[S], D1[S];
            const TIn x = xv[q][u];
            if constexpr (BOTH) {
              // 2^(8-e) as pre * scale: rows below 2^-119 would overflow a single FP32
              // power of two, so they are first lifted by 2^64 (exact)
              const bool tiny = e < -118;
              const float pre = tiny ? 18446744073709551616.0f : 1.0f;
              const float scale = __int_as_float((127 + 8 - (tiny ? e + 64 : e)) << 23);
              // B' real layout (Re, -Im) for B items; A as (Re, Im)
              float2 v = __fmul2_rn(make_float2(x.x, isA ? x.y : -x.y), make_float2(pre, pre));
              float2 D[S];
              digits_f32x2<S>(v, scale, D);
#pragma unroll
              for (int s2 = 0; s2 < S; ++s2) {
                packed[s2][u] = pack_pair(D[s2]);
                packed2[s2][u] = pack_pair(make_float2(D[s2].y, D[s2].x)) ^ 0x80000000u;
              }
            } else if constexpr (sizeof(TIn) == 8) {
              const bool tiny = e < -118;
              const float pre = tiny ? 18446744073709551616.0f : 1.0f;
              const float scale = __int_as_float((127 + 8 - (tiny ? e + 64 : e)) << 23);
              float v0 = x.x * pre, v1 = x.y * pre;
              if (!isA) {
                if (part == 0) v1 = -v1;
                else { v0 = x.y; v1 = x.x; }
              }
              digits_f32<S>(v0, scale, D0);
              digits_f32<S>(v1, scale, D1);
            } else {
              double v0 = x.x, v1 = x.y;
              if (!isA) {
                if (part == 0) v1 = __longlong_as_double(__double_as_longlong(v1) ^ (1ll << 63));
                else { v0 = x.y; v1 = x.x; }
              }
              digits_f64<S>(v0, e, D0);
              digits_f64<S>(v1, e, D1);
            }
            if constexpr (!BOTH) {
#pragma unroll
              for (int s2 = 0; s2 < S; ++s2) packed[s2][u] = pack_bf16x2(D0[s2], D1[s2]);
            }
          }
          // canonical no-swizzle K-major: (r/8)*SBO + g*LBO + (r%8)*16
          const uint32_t off = (uint32_t)((r >> 3) * SBO + g * LBO + (r & 7) * 16);
          unsigned char* base = isA ? stA : stB;
          const int pstride = isA ? PLANE_BYTES : BPLANE;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2)
            *reinterpret_cast<uint4*>(base + (size_t)s2 * pstride + off) =
                make_uint4(packed[s2][0], packed[s2][1], packed[s2][2], packed[s2][3]);
          if constexpr (BOTH) {
            if (isA) {
#pragma unroll
              for (int s2 = 0; s2 < S; ++s2)
                *reinterpret_cast<uint4*>(base + (size_t)(S + s2) * PLANE_BYTES + off) =
                    make_uint4(packed2[s2][0], packed2[s2][1], packed2[s2][2], packed2[s2][3]);
            }
          }
        }
        fence_proxy_async();
        mbar_arrive(&full[st]);
      }
      ++proc;
    }
  } else if (warp == MMA_WARP) {
    // ======================== MMA issuer (one thread)
    if (lane == 0) {
      const uint32_t idesc = make_idesc(128, NT);
      uint32_t proc = 0, gchunk = 0;
      for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
        const long long b = w / (NPARTS == 2 ? ntile : 2 * ntile);
        if (a.active && !a.active[b]) continue;
        if (!mbar_wait(tmem_empty, (proc & 1) ^ 1, abort_flag, tcount)) break;
        tc_fence_after();
        uint32_t touched = 0;
        for (int c = 0; c < nch; ++c, ++gchunk) {
          const int st = gchunk % stages;
          const uint32_t ph = (gchunk / stages) & 1;
          if (!mbar_wait(&full[st], ph, abort_flag, tcount)) break;
          tc_fence_after();
          const uint32_t sA = smem_u32(tiles + (size_t)st * stage_bytes);
          const uint32_t sB = sA + APLANES * S * PLANE_BYTES;
#pragma unroll
          for (int kk = 0; kk < KC / 16; ++kk) {
#pragma unroll
            for (int pp = 0; pp < NPARTS; ++pp) {
#pragma unroll
              for (int s = 0; s < S; ++s) {
#pragma unroll
                for (int t = 0; t < S; ++t) {
                  if (s + t > L) continue;
                  const int acc = pp * NACC + ((s + t) < NACC - 1 ? (s + t) : NACC - 1);
                  const uint64_t ad = make_desc(sA + (pp * S + s) * PLANE_BYTES + kk * 2 * LBO);
                  const uint64_t bd = make_desc(sB + t * BPLANE + kk * 2 * LBO);
                  umma(tmem + acc * NT, ad, bd, idesc, (touched >> acc) & 1);
                  touched |= 1u << acc;
                }
              }
            }
          }
          umma_commit(&empty[st]);
        }
        umma_commit(tmem_full);
        ++proc;
      }
      // drain: wait until every MMA issued by this thread has completed
      umma_commit(drain);
      int dummy = 0;
      volatile int* never = &dummy;
      mbar_wait(drain, 0, never, tcount);
    }
    __syncwarp();
  } else {
    // ======================== epilogue (warps 0..3 own TMEM lanes 0..127)
    const int row = warp * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t proc = 0;
    for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
      const long long b = w / (NPARTS == 2 ? ntile : 2 * ntile);
      const int part0 = BOTH ? 0 : (int)((w / ntile) & 1), ct = (int)(w % ntile);
      if (a.active && !a.active[b]) continue;
      if (!mbar_wait(tmem_full, proc & 1, abort_flag, tcount)) break;
      const int* erow = a.scales + b * 256;
      const int* fcol = erow + 128;
      tc_fence_after();
      void* C = batch_ptr<TOut>(a.C, b);
      const void* D = a.D.p ? batch_ptr<const TOut>(a.D, b) : nullptr;
      const int ei = erow[row];
      const float alpha = (float)a.alpha_re, beta = (float)a.beta_re;
      // columns per TMEM read (register budget of the wider 128-column CTAs)
      constexpr int CW = (NACC > 4 || NPROD > 256) ? 8 : 16;
      for (int pp = 0; pp < NPARTS; ++pp) {
      const int part = BOTH ? pp : part0;
      double zpart = 0.0;
      if (a.Z.p) {
        const double2 z = *batch_ptr<const double2>(a.Z, b);
        zpart = part ? z.y : z.x;
      }
      for (int j0 = 0; j0 < NT; j0 += CW) {
        uint32_t r[NACC][16];
#pragma unroll
        for (int acc = 0; acc < NACC; ++acc) {
          const uint32_t col = (uint32_t)((pp * NACC + acc) * NT + j0);
          if constexpr (CW == 16) tmem_ld16(lane_base + col, r[acc]);
          else tmem_ld8(lane_base + col, r[acc]);
        }
        tmem_wait_ld();
        if (row < m) {
#pragma unroll
          for (int jj = 0; jj < CW; ++jj) {
            const int j = ct * NT + j0 + jj;
            if (j < n) {
              float hi = __uint_as_float(r[0][jj]), lo = 0.f, e;
#pragma unroll
              for (int acc = 1; acc < NACC; ++acc) {
                float s;
                two_sum(hi, __uint_as_float(r[acc][jj]), s, e);
                hi = s;
                lo += e;
              }
              float s2;
              two_sum(hi, lo, s2, e);  // normalise: |lo| <= ulp(hi)/2
              const int e2 = ei + fcol[j] - 16;
              Store<TOut>::put(C, row + (long long)j * a.C.ld, part, s2, e, e2, alpha, beta, D,
                               row + (long long)j * a.D.ld, row == j && a.Z.p, zpart);
            }
          }
        }
      }
      }  // parts
      tc_fence_before();
      mbar_arrive(tmem_empty);
      ++proc;
    }
  }
  // ---- teardown: every MMA has completed (drained above); free TMEM
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == MMA_WARP) {
    tc::tmem_dealloc(tmem, 512);
  }
}

template <int S, int L, int NT, typename TIn, typename TOut>
cudaError_t launch(const GemmArgs& a, cudaStream_t s) {
  int dev = 0, sms = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  constexpr int aplanes = sizeof(TIn) == 8 ? 2 : 1;  // complex64: both parts per item
  const int stage_bytes = S * (aplanes * PLANE_BYTES + NT * KC * 2);
  const int extra = 2048 + 8 * 64 + 64;  // barriers + exponents + tmem slot
  int stages = (maxsm - extra) / stage_bytes;
  if (stages > 4) stages = 4;
  if (stages < 2) return cudaErrorInvalidConfiguration;
  const size_t smem = (size_t)stages * stage_bytes + extra;
  cudaError_t e = cudaFuncSetAttribute(zgemm_oz_kernel<S, L, NT, TIn, TOut>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int ntile = (((a.n + 15) & ~15) + NT - 1) / NT;
  const long long items = (sizeof(TIn) == 8 ? 1LL : 2LL) * ntile * a.batch;
  const int grid = (int)(items < sms ? items : sms);
  if (!a.scales) return cudaErrorInvalidValue;
  const long long gb = a.batch < 65535 ? a.batch : 65535;
  oz_scales_kernel<TIn><<<dim3((unsigned)gb, 2), 256, 0, s>>>(a);
  count_launch();
  zgemm_oz_kernel<S, L, NT, TIn, TOut><<<grid, Roles<NT>::NTHREADS, smem, s>>>(a, stages);
  count_launch();
  return cudaGetLastError();
}


// ============================================================ TMA-fed complex64 product
// The complex64 sweep's product C = alpha op(A) op(B) + beta D + z I (S = 4 digits, levels
// <= 3) with its operands staged by the tensor memory accelerator:
//  * a loader thread copies each stage's raw complex64 tiles -- op(A) 128 rows x 8 complex
//    k and op(B) 8 k x 128 columns -- from global memory into a ring of RSTAGES shared-memory
//    slots with cp.async.bulk.tensor (3-D tensor maps over (floats, vectors, batch entry));
//  * producer warps split the raw tiles, shared memory to shared memory, into the digit
//    planes of A' = (Re, Im) op(A) and of the two layouts of op(B), B'_r = (Re, -Im) and
//    B'_i = (Im, Re), so that Re C = A' B'_r and Im C = A' B'_i, and fence each slot's reads
//    against the async proxy before handing the slot back to the loader;
//  * a work item is a whole product (n <= 128): both real parts of all columns, so every
//    MMA is 128 x 128 x 16 and op(A) is split once per product.  The four accumulators (two
//    parts x level 0 / levels 1-3) take all 512 TMEM columns; eight epilogue warps (two per
//    TMEM lane quarter, one column half each) keep the unoverlapped epilogue short.
// A tile that is contiguous along rows (op(A) = N, op(B) = C) is copied as [k][row]; one
// that is contiguous along k (op(A) = C, op(B) = N) as [row][k] in 64-byte rows under the
// 64-byte swizzle, so that the producers' 16-byte reads down a column of rows spread over
// the banks.  The epilogue's arithmetic is the register-staged kernel's: the two kernels
// give the same bits.
namespace c64t {
constexpr int S = 4, L = 3;              // digits, highest level kept
constexpr int NT = 128;                  // output columns per item (all of them)
constexpr int KCC = 8;                   // complex k per stage (16 real K: one MMA K step)
constexpr int DSTAGES = 3, RSTAGES = 5;  // digit stages, raw (TMA) stages
constexpr int NEPI = 256;                // epilogue threads (8 warps)
constexpr int NPROD = 256;               // producer threads (8 warps)
constexpr int PROD_WARP0 = NEPI / 32, LOAD_WARP = PROD_WARP0 + NPROD / 32, MMA_WARP = LOAD_WARP + 1;
constexpr int NTHREADS = 32 * (MMA_WARP + 1);
constexpr int PLANE = 128 * 2 * KCC * 2;  // one digit plane: 128 rows x 16 BF16 (4 KB)
constexpr int DSTAGE = 3 * S * PLANE;     // A', B'_r, B'_i: 48 KB
constexpr int RAW_A = 128 * KCC * 8, RAW_B = NT * KCC * 8;  // 8 KB, 8 KB
constexpr int RSTAGE = RAW_A + RAW_B;
constexpr uint32_t SBO_T = (2 * KCC / 8) * 128;  // 8-row groups of a digit plane (256 B)
constexpr int SMEM = 1024 + RSTAGES * RSTAGE + DSTAGES * DSTAGE + 256;
static_assert(SMEM <= 232448, "shared memory");
static_assert(RAW_A % 1024 == 0 && RSTAGE % 1024 == 0, "swizzled boxes need 1 KB alignment");

// operand tile layout in a raw slot
enum { MN_MAJOR = 0, K_MAJOR = 1 };

struct Args {
  GemmArgs g;
  int layoutA, layoutB;  // MN_MAJOR / K_MAJOR
};

// complex elements 4g .. 4g+3 (g = 0, 1) of vector v of a raw tile of 8 complex k:
// MN-major [kc][v] (128 vectors), K-major [v][kc] in 64-byte rows under the 64-byte swizzle
// (16-byte chunk c of row v at chunk c ^ ((v >> 1) & 3))
__device__ __forceinline__ void raw_read4(const unsigned char* base, int layout, int v, int g,
                                          float2* x) {
  if (layout == MN_MAJOR) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
      x[u] = *reinterpret_cast<const float2*>(base + ((size_t)(4 * g + u) * 128 + v) * 8);
  } else {
    const int sw = (v >> 1) & 3;
    const float4 p0 = *reinterpret_cast<const float4*>(base + v * 64 + (((2 * g) ^ sw) << 4));
    const float4 p1 = *reinterpret_cast<const float4*>(base + v * 64 + (((2 * g + 1) ^ sw) << 4));
    x[0] = make_float2(p0.x, p0.y);
    x[1] = make_float2(p0.z, p0.w);
    x[2] = make_float2(p1.x, p1.y);
    x[3] = make_float2(p1.z, p1.w);
  }
}

// 2^(8-e) as pre * scale: vectors below 2^-119 would overflow one FP32 power of two, so they
// are first lifted by 2^64 (exact).  sign = -1 conjugates (op = C).
__device__ __forceinline__ void digit_scale(int e, float sign, float2& m, float& sc) {
  const bool tiny = e < -118;
  const float pre = tiny ? 18446744073709551616.0f : 1.0f;
  m = make_float2(pre, pre * sign);
  sc = __int_as_float((127 + 8 - (tiny ? e + 64 : e)) << 23);
}
// both real parts of an output element from their accumulators (level 0, levels 1-3),
// with the arithmetic of Store<float2>::put lane by lane in packed FP32x2 operations (each
// lane rounds exactly as the scalar form: the same bits in half the instructions):
// normalised (hi, lo) by two TwoSums, scaled by 2^e2 and alpha, beta d and z added
__device__ __forceinline__ float2 fsub2(float2 x, float2 y) {  // x - y, exact as a subtraction
  return __ffma2_rn(y, make_float2(-1.0f, -1.0f), x);
}
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = fsub2(s, a);
  e = __fadd2_rn(fsub2(a, fsub2(s, bb)), fsub2(b, bb));
}
__device__ __forceinline__ float2 c64_pair(uint32_t r0, uint32_t r1, uint32_t i0, uint32_t i1,
                                           int e2, float alpha, float beta, const float2* d,
                                           bool diag, double2 z) {
  float2 hi, lo, s2, e;
  two_sum2(make_float2(__uint_as_float(r0), __uint_as_float(i0)),
           make_float2(__uint_as_float(r1), __uint_as_float(i1)), hi, lo);
  two_sum2(hi, lo, s2, e);
  float2 v, w;
  const float2 al = make_float2(alpha, alpha);
  if (e2 > -126 && e2 < 128) {
    const float sc = __int_as_float((127 + e2) << 23);  // 2^e2
    v = __fmul2_rn(al, __fmul2_rn(s2, make_float2(sc, sc)));
    w = __fmul2_rn(al, __fmul2_rn(e, make_float2(sc, sc)));
  } else {
    v = make_float2(alpha * ldexpf(s2.x, e2), alpha * ldexpf(s2.y, e2));
    w = make_float2(alpha * ldexpf(e.x, e2), alpha * ldexpf(e.y, e2));
  }
  if (d) v = __ffma2_rn(make_float2(beta, beta), *d, v);
  if (diag) v = __fadd2_rn(v, make_float2((float)z.x, (float)z.y));
  return __fadd2_rn(v, w);
}

__global__ void __launch_bounds__(NTHREADS, 1)
    zgemm_c64_tma_kernel(const __grid_constant__ Args args, const __grid_constant__ CUtensorMap tmA,
                          const __grid_constant__ CUtensorMap tmB) {
  const GemmArgs& a = args.g;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char* raw = smem;
  unsigned char* dig = smem + (size_t)RSTAGES * RSTAGE;
  uint64_t* bars = reinterpret_cast<uint64_t*>(dig + (size_t)DSTAGES * DSTAGE);
  uint64_t* dfull = bars;
  uint64_t* dempty = dfull + DSTAGES;
  uint64_t* rfull = dempty + DSTAGES;
  uint64_t* rempty = rfull + RSTAGES;
  uint64_t* tfull = rempty + RSTAGES;
  uint64_t* tempty = tfull + 1;
  uint64_t* drain = tempty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  int* const tcount = a.timeouts ? a.timeouts : &g_oz_timeouts;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = a.m, n = a.n, K = a.k;
  const int nch = (K + KCC - 1) / KCC;
  const long long nitems = a.batch;

  if (tid == 0) {
    for (int s = 0; s < DSTAGES; ++s) { mbar_init(&dfull[s], NPROD); mbar_init(&dempty[s], 1); }
    for (int s = 0; s < RSTAGES; ++s) { mbar_init(&rfull[s], 1); mbar_init(&rempty[s], NPROD); }
    mbar_init(tfull, 1);
    mbar_init(tempty, NEPI);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP) tc::tmem_alloc(tmem_slot, 512);
  if (warp == LOAD_WARP && lane == 0) {
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == LOAD_WARP) {
    if (lane == 0) {
      uint32_t g = 0;
      uint32_t pend_parity[RSTAGES];
      bool pend[RSTAGES];
#pragma unroll
      for (int s = 0; s < RSTAGES; ++s) { pend[s] = false; pend_parity[s] = 0; }
      for (long long b = blockIdx.x; b < nitems && !*abort_flag; b += gridDim.x) {
        if (a.active && !a.active[b]) continue;
        const int ea = a.A.stride == 0 ? 0 : (int)batch_index(a.A, b);
        const int eb = a.B.stride == 0 ? 0 : (int)batch_index(a.B, b);
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++g) {
          const int slot = (int)(g % RSTAGES);
          const uint32_t ph = (g / RSTAGES) & 1;
          if (!mbar_wait(&rempty[slot], ph ^ 1, abort_flag, tcount)) { ok = false; break; }
          unsigned char* dA = raw + (size_t)slot * RSTAGE;
          unsigned char* dB = dA + RAW_A;
          tc::mbar_arrive_expect_tx(&rfull[slot], RSTAGE);
          const int k0 = c * KCC;
          if (args.layoutA == MN_MAJOR) tc::tma_load_3d(dA, &tmA, 0, k0, ea, &rfull[slot]);
          else tc::tma_load_3d(dA, &tmA, 2 * k0, 0, ea, &rfull[slot]);
          if (args.layoutB == MN_MAJOR) tc::tma_load_3d(dB, &tmB, 0, k0, eb, &rfull[slot]);
          else tc::tma_load_3d(dB, &tmB, 2 * k0, 0, eb, &rfull[slot]);
          pend[slot] = true;
          pend_parity[slot] = ph;
        }
        if (!ok) break;
      }
      int zero = 0;
      volatile int* never = &zero;
      for (int s = 0; s < RSTAGES; ++s)
        if (pend[s]) mbar_wait(&rfull[s], pend_parity[s], never, tcount);
    }
    __syncwarp();
  } else if (warp >= PROD_WARP0 && warp < LOAD_WARP) {
    // thread p: row r of op(A) and column r of op(B), 4-k group g
    const int p = tid - NEPI;
    const int r = p & 127, g4 = p >> 7;
    const uint32_t off = (uint32_t)((r >> 3) * SBO_T + g4 * 128 + (r & 7) * 16);
    const float sgnA = a.opA == OP_C ? -1.f : 1.f, sgnB = a.opB == OP_C ? -1.f : 1.f;
    uint32_t g = 0;
    for (long long b = blockIdx.x; b < nitems && !*abort_flag; b += gridDim.x) {
      if (a.active && !a.active[b]) continue;
      const int* erow = a.scales + b * 256;
      float2 mA, mB;
      float scA, scB;
      digit_scale(r < m ? erow[r] : 0, sgnA, mA, scA);
      digit_scale(r < n ? erow[128 + r] : 0, sgnB, mB, scB);
      bool ok = true;
      for (int c = 0; c < nch; ++c, ++g) {
        const int rs = (int)(g % RSTAGES), ds = (int)(g % DSTAGES);
        if (!mbar_wait(&rfull[rs], (g / RSTAGES) & 1, abort_flag, tcount)) { ok = false; break; }
        const unsigned char* rA = raw + (size_t)rs * RSTAGE;
        float2 xa[4], xb[4];
        raw_read4(rA, args.layoutA, r, g4, xa);
        raw_read4(rA + RAW_A, args.layoutB, r, g4, xb);
        fence_proxy_async();
        mbar_arrive(&rempty[rs]);
        if (!mbar_wait(&dempty[ds], ((g / DSTAGES) & 1) ^ 1, abort_flag, tcount)) {
          ok = false;
          break;
        }
        unsigned char* dA = dig + (size_t)ds * DSTAGE;
        unsigned char* dBr = dA + S * PLANE;
        unsigned char* dBi = dBr + S * PLANE;
        uint32_t pa[S][4], pr[S][4], pi[S][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float2 D[S];
          digits_f32x2<S>(__fmul2_rn(xa[u], mA), scA, D);
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2) pa[s2][u] = pack_pair(D[s2]);
          digits_f32x2<S>(__fmul2_rn(xb[u], mB), scB, D);
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2) {
            pr[s2][u] = pack_pair(D[s2]) ^ 0x80000000u;
            pi[s2][u] = __byte_perm(__float_as_uint(D[s2].x), __float_as_uint(D[s2].y), 0x3276);
          }
        }
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
          *reinterpret_cast<uint4*>(dA + (size_t)s2 * PLANE + off) =
              make_uint4(pa[s2][0], pa[s2][1], pa[s2][2], pa[s2][3]);
          *reinterpret_cast<uint4*>(dBr + (size_t)s2 * PLANE + off) =
              make_uint4(pr[s2][0], pr[s2][1], pr[s2][2], pr[s2][3]);
          *reinterpret_cast<uint4*>(dBi + (size_t)s2 * PLANE + off) =
              make_uint4(pi[s2][0], pi[s2][1], pi[s2][2], pi[s2][3]);
        }
        fence_proxy_async();
        mbar_arrive(&dfull[ds]);
      }
      if (!ok) break;
    }
  } else if (warp == MMA_WARP) {
    // TMEM columns: [128 (2 part + level class)]: Re level 0, Re 1-3, Im level 0, Im 1-3
    if (lane == 0) {
      const uint32_t idesc = make_idesc(128, NT);
      uint32_t g = 0, li = 0;
      for (long long b = blockIdx.x; b < nitems && !*abort_flag; b += gridDim.x) {
        if (a.active && !a.active[b]) continue;
        if (!mbar_wait(tempty, (li & 1) ^ 1, abort_flag, tcount)) break;
        tc_fence_after();
        uint32_t touched = 0;
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++g) {
          const int ds = (int)(g % DSTAGES);
          if (!mbar_wait(&dfull[ds], (g / DSTAGES) & 1, abort_flag, tcount)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sA = smem_u32(dig + (size_t)ds * DSTAGE);
          const uint32_t sB = sA + S * PLANE;
#pragma unroll
          for (int part = 0; part < 2; ++part) {
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2) {
#pragma unroll
              for (int t = 0; t < S; ++t) {
                if (s2 + t > L) continue;
                const int acc = 2 * part + (s2 + t > 0 ? 1 : 0);
                const uint64_t ad = tc::make_desc(sA + s2 * PLANE, 128, SBO_T);
                const uint64_t bd = tc::make_desc(sB + (part * S + t) * PLANE, 128, SBO_T);
                umma(tmem + (uint32_t)(acc * NT), ad, bd, idesc, (touched >> acc) & 1);
                touched |= 1u << acc;
              }
            }
          }
          umma_commit(&dempty[ds]);
        }
        if (!ok) break;
        umma_commit(tfull);
        ++li;
      }
      umma_commit(drain);
      int zero = 0;
      volatile int* never = &zero;
      mbar_wait(drain, 0, never, tcount);
    }
    __syncwarp();
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. (rows) for columns 64 (w / 4) ..
    const int row = (warp & 3) * 32 + lane, half = warp >> 2;
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const float alpha = (float)a.alpha_re, beta = (float)a.beta_re;
    uint32_t li = 0;
    for (long long b = blockIdx.x; b < nitems && !*abort_flag; b += gridDim.x) {
      if (a.active && !a.active[b]) continue;
      if (!mbar_wait(tfull, li & 1, abort_flag, tcount)) break;
      tc_fence_after();
      const int* erow = a.scales + b * 256;
      const int* fcol = erow + 128;
      float2* C = batch_ptr<float2>(a.C, b);
      const float2* D = a.D.p ? batch_ptr<const float2>(a.D, b) : nullptr;
      double2 z = make_double2(0.0, 0.0);
      if (a.Z.p) z = *batch_ptr<const double2>(a.Z, b);
      const int ei = erow[row];
#pragma unroll 1
      for (int j0 = half * 64; j0 < half * 64 + 64; j0 += 16) {
        uint32_t v[4][16];
#pragma unroll
        for (int q = 0; q < 4; ++q) tmem_ld16(lane_base + (uint32_t)(q * NT + j0), v[q]);
        tmem_wait_ld();
        if (row < m) {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            const int jcol = j0 + jj;
            if (jcol < n) {
              const float2* d = D ? D + row + (long long)jcol * a.D.ld : nullptr;
              C[row + (long long)jcol * a.C.ld] =
                  c64_pair(v[0][jj], v[1][jj], v[2][jj], v[3][jj], ei + fcol[jcol] - 16,
                                 alpha, beta, d, a.Z.p && row == jcol, z);
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(tempty);
      ++li;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == MMA_WARP) tc::tmem_dealloc(tmem, 512);
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, looked up once through the runtime (no -lcuda)
EncodeTiled encode_tiled() {
  static EncodeTiled fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<EncodeTiled>(nullptr);
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// 3-D tensor map (floats, vectors or k, batch entry) of one complex64 operand: boxes of 8
// complex k x 128 vectors; K-major boxes (64-byte rows) take the 64-byte swizzle.  A batch
// reference qualifies when a tensor map can address it: no index array, a 16-byte aligned
// base, and even leading dimension and batch stride (16-byte strides).
bool make_map(CUtensorMap* map, const BatchRef& R, int layout, int vecs, int K, long long batch) {
  const EncodeTiled fn = encode_tiled();
  if (!fn || !R.p || R.idx || (reinterpret_cast<uintptr_t>(R.p) & 15) || (R.ld & 1) ||
      (R.stride & 1) || R.ld < (layout == MN_MAJOR ? vecs : K))
    return false;
  const cuuint64_t ldb = (cuuint64_t)R.ld * 8;
  cuuint64_t dims[3], strides[2];
  cuuint32_t box[3], es[3] = {1, 1, 1};
  if (layout == MN_MAJOR) {
    dims[0] = 2 * (cuuint64_t)vecs; dims[1] = K;
    box[0] = 2 * 128; box[1] = KCC;
  } else {
    dims[0] = 2 * (cuuint64_t)K; dims[1] = vecs;
    box[0] = 2 * KCC; box[1] = 128;
  }
  box[2] = 1;
  const long long entries = R.stride == 0 ? 1 : (R.mod > 0 ? R.mod : batch);
  dims[2] = (cuuint64_t)entries;
  strides[0] = ldb;
  strides[1] = R.stride == 0 ? ((ldb * dims[1] + 15) & ~(cuuint64_t)15)
                             : (cuuint64_t)R.stride * 8;
  if (strides[1] < ldb * dims[1]) return false;
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, R.p, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE,
            layout == K_MAJOR ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launches the TMA-fed product when both operands qualify; *used = false otherwise (the
// caller then runs the register-staged kernel).
cudaError_t launch(const GemmArgs& g, cudaStream_t s, bool* used) {
  *used = false;
  Args args;
  args.g = g;
  args.layoutA = g.opA == OP_N ? MN_MAJOR : K_MAJOR;
  args.layoutB = g.opB == OP_N ? K_MAJOR : MN_MAJOR;
  alignas(64) CUtensorMap ma, mb;
  if (!make_map(&ma, g.A, args.layoutA, g.m, g.k, g.batch) ||
      !make_map(&mb, g.B, args.layoutB, g.n, g.k, g.batch))
    return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaFuncSetAttribute(zgemm_c64_tma_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
  if (e != cudaSuccess) return e;
  const long long gb = g.batch < 65535 ? g.batch : 65535;
  oz_scales_kernel<float2><<<dim3((unsigned)gb, 2), 256, 0, s>>>(g);
  count_launch();
  const int grid = (int)(g.batch < sms ? g.batch : sms);
  zgemm_c64_tma_kernel<<<grid, NTHREADS, SMEM, s>>>(args, ma, mb);
  count_launch();
  *used = true;
  return cudaGetLastError();
}
}  // namespace c64t

// ============================================================ TMA-fed complex128 product
// The FP64-grade split product (complex128 blocks; S = 7 digits for the leads, 6 for the
// complex128 sweep, 4 for refinement updates) with the operands staged by the tensor
// memory accelerator, as the complex64 product above: raw complex128 tiles (op(A) 128 rows
// x 8 complex k, op(B) 8 k x 64 columns) arrive in a ring of shared-memory slots by
// cp.async.bulk.tensor, producer warps split them shared memory to shared memory into the
// digit planes (integer digit extraction of the FP64 values), one MMA warp issues every
// digit pair, and the epilogue assembles FP64 results from the per-level accumulators.
// A work item is one real part of one 64-column tile; every level keeps its own (exact)
// accumulator, NACC = S accumulators x 64 columns of TMEM.  complex128 strides are always
// multiples of 16 bytes, so every operand qualifies for a tensor map.
namespace c128t {
constexpr int NT = 64;                   // output columns per item
constexpr int KCC = 8;                   // complex k per stage (16 real K: one MMA K step)
constexpr int DSTAGES = 3, RSTAGES = 4;  // digit stages, raw (TMA) stages
constexpr int NPROD = 384;               // producer threads: one (row/column, 4-k group) each
constexpr int LOAD_WARP = 4 + NPROD / 32, MMA_WARP = LOAD_WARP + 1;
constexpr int NTHREADS = 32 * (MMA_WARP + 1);
constexpr int APLANE = 128 * 2 * KCC * 2;  // one digit plane of A': 128 rows x 16 BF16 (4 KB)
constexpr int BPLANE = NT * 2 * KCC * 2;   // one digit plane of B': 64 rows (2 KB)
constexpr int RAW_A = 128 * KCC * 16, RAW_B = NT * KCC * 16;  // 16 KB, 8 KB
constexpr int RSTAGE = RAW_A + RAW_B;
constexpr uint32_t SBO_T = (2 * KCC / 8) * 128;  // 8-row groups of a digit plane (256 B)
template <int S> struct Cfg {
  static constexpr int NACC = S;  // levels 0 .. S-1, one exact accumulator each
  // Two accumulator sets where they fit the 512 TMEM columns (the 4-digit product): the
  // epilogue of one item then runs while the next item's products are issued.
  static constexpr int NBUF = 2 * NACC * NT <= 512 ? 2 : 1;
  static constexpr int DSTAGE = S * (APLANE + BPLANE);
  static constexpr int SMEM = 1024 + RSTAGES * RSTAGE + DSTAGES * DSTAGE + 256;
  static_assert(SMEM <= 232448, "shared memory");
};
static_assert(RAW_A % 1024 == 0 && RSTAGE % 1024 == 0, "swizzled boxes need 1 KB alignment");

enum { MN_MAJOR = 0, K_MAJOR = 1 };

struct Args {
  GemmArgs g;
  int layoutA, layoutB;
};

// complex element (v, kc) of a raw tile: MN-major tiles hold [kc][v] (vecs vectors),
// K-major tiles [v][kc] in 128-byte swizzled rows (one complex per 16-byte chunk)
__device__ __forceinline__ double2 raw_elem(const unsigned char* base, int layout, int v, int kc,
                                            int vecs) {
  if (layout == MN_MAJOR)
    return *reinterpret_cast<const double2*>(base + ((size_t)kc * vecs + v) * 16);
  return *reinterpret_cast<const double2*>(base + v * 128 + ((kc ^ (v & 7)) << 4));
}
__device__ __forceinline__ double dneg(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (1ll << 63));
}

template <int S>
__global__ void __launch_bounds__(NTHREADS, 1)
    zgemm_c128_tma_kernel(const __grid_constant__ Args args,
                          const __grid_constant__ CUtensorMap tmA,
                          const __grid_constant__ CUtensorMap tmB) {
  constexpr int L = S - 1, NACC = Cfg<S>::NACC, NBUF = Cfg<S>::NBUF;
  constexpr int DSTAGE = Cfg<S>::DSTAGE;
  const GemmArgs& a = args.g;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char* raw = smem;                               // [RSTAGES][A tile | B tile]
  unsigned char* dig = smem + (size_t)RSTAGES * RSTAGE;    // [DSTAGES][A' planes | B' planes]
  uint64_t* bars = reinterpret_cast<uint64_t*>(dig + (size_t)DSTAGES * DSTAGE);
  uint64_t* dfull = bars;
  uint64_t* dempty = dfull + DSTAGES;
  uint64_t* rfull = dempty + DSTAGES;
  uint64_t* rempty = rfull + RSTAGES;
  uint64_t* tfull = rempty + RSTAGES;  // [NBUF]
  uint64_t* tempty = tfull + 2;        // [NBUF]
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  int* const tcount = a.timeouts ? a.timeouts : &g_oz_timeouts;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m = a.m, n = a.n, K = a.k;
  const int nch = (K + KCC - 1) / KCC;
  const int ntile = (n + NT - 1) / NT;
  // item w: batch entry w / (2 ntile), real part (w / ntile) % 2, column tile w % ntile
  const long long nitems = 2LL * ntile * a.batch;

  if (tid == 0) {
    for (int s = 0; s < DSTAGES; ++s) { mbar_init(&dfull[s], NPROD); mbar_init(&dempty[s], 1); }
    for (int s = 0; s < RSTAGES; ++s) { mbar_init(&rfull[s], 1); mbar_init(&rempty[s], NPROD); }
    for (int s = 0; s < NBUF; ++s) { mbar_init(&tfull[s], 1); mbar_init(&tempty[s], 128); }
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP) tc::tmem_alloc(tmem_slot, 512);
  if (warp == LOAD_WARP && lane == 0) {
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == LOAD_WARP) {
    // ======================== loader
    if (lane == 0) {
      uint32_t g = 0;
      uint32_t pend_parity[RSTAGES];
      bool pend[RSTAGES];
#pragma unroll
      for (int s = 0; s < RSTAGES; ++s) { pend[s] = false; pend_parity[s] = 0; }
      for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
        const long long b = w / (2 * ntile);
        const int ct = (int)(w % ntile);
        if (a.active && !a.active[b]) continue;
        const int ea = a.A.stride == 0 ? 0 : (int)batch_index(a.A, b);
        const int eb = a.B.stride == 0 ? 0 : (int)batch_index(a.B, b);
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++g) {
          const int slot = (int)(g % RSTAGES);
          const uint32_t ph = (g / RSTAGES) & 1;
          if (!mbar_wait(&rempty[slot], ph ^ 1, abort_flag, tcount)) { ok = false; break; }
          unsigned char* dA = raw + (size_t)slot * RSTAGE;
          unsigned char* dB = dA + RAW_A;
          tc::mbar_arrive_expect_tx(&rfull[slot], RSTAGE);
          const int k0 = c * KCC;
          if (args.layoutA == MN_MAJOR) tc::tma_load_3d(dA, &tmA, 0, k0, ea, &rfull[slot]);
          else tc::tma_load_3d(dA, &tmA, 2 * k0, 0, ea, &rfull[slot]);
          if (args.layoutB == MN_MAJOR) tc::tma_load_3d(dB, &tmB, 2 * ct * NT, k0, eb, &rfull[slot]);
          else tc::tma_load_3d(dB, &tmB, 2 * k0, ct * NT, eb, &rfull[slot]);
          pend[slot] = true;
          pend_parity[slot] = ph;
        }
        if (!ok) break;
      }
      int zero = 0;
      volatile int* never = &zero;
      for (int s = 0; s < RSTAGES; ++s)
        if (pend[s]) mbar_wait(&rfull[s], pend_parity[s], never, tcount);
    }
    __syncwarp();
  } else if (warp >= 4 && warp < LOAD_WARP) {
    // ======================== producers: one (row or column, 4-k group) per thread:
    // p < 256: row p & 127 of op(A), group p >> 7; else column q & 63 of op(B), group q >> 6
    const int p = tid - 128;
    const bool isA = p < 256;
    const int q = isA ? p : p - 256;
    const int v = isA ? (q & 127) : (q & (NT - 1)), gq = isA ? (q >> 7) : (q / NT);
    const uint32_t off = (uint32_t)((v >> 3) * SBO_T + gq * 128 + (v & 7) * 16);
    const int layout = isA ? args.layoutA : args.layoutB;
    const int conj = isA ? (a.opA == OP_C) : (a.opB == OP_C);
    uint32_t g = 0;
    for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
      const long long b = w / (2 * ntile);
      const int part = (int)((w / ntile) & 1), ct = (int)(w % ntile);
      if (a.active && !a.active[b]) continue;
      const int* erow = a.scales + b * 256;
      const int vg = isA ? v : ct * NT + v;  // row of op(A) / column of op(B)
      const int e = isA ? (vg < m ? erow[vg] : 0) : (vg < n ? erow[128 + vg] : 0);
      bool ok = true;
      for (int c = 0; c < nch; ++c, ++g) {
        const int rs = (int)(g % RSTAGES), ds = (int)(g % DSTAGES);
        if (!mbar_wait(&rfull[rs], (g / RSTAGES) & 1, abort_flag, tcount)) { ok = false; break; }
        const unsigned char* rt = raw + (size_t)rs * RSTAGE + (isA ? 0 : RAW_A);
        double2 x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = raw_elem(rt, layout, v, 4 * gq + u, isA ? 128 : NT);
        // release the slot to the next cp.async.bulk.tensor only after a proxy fence: the
        // mbarrier orders these generic-proxy reads for the loader thread, not for the
        // async-proxy write that follows, which could otherwise land before them
        fence_proxy_async();
        mbar_arrive(&rempty[rs]);
        if (!mbar_wait(&dempty[ds], ((g / DSTAGES) & 1) ^ 1, abort_flag, tcount)) {
          ok = false;
          break;
        }
        uint32_t pk[S][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          // A' = (Re, Im) of op(A); B' = (Re, -Im) (real part of C) or (Im, Re) (imaginary)
          // of op(B); op = C conjugates; negating an FP64 value is exact
          double v0 = x[u].x, v1 = conj ? dneg(x[u].y) : x[u].y;
          if (!isA) {
            if (part == 0) v1 = dneg(v1);
            else { const double t = v0; v0 = v1; v1 = t; }
          }
          float D0[S], D1[S];
          digits_f64<S>(v0, e, D0);
          digits_f64<S>(v1, e, D1);
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2) pk[s2][u] = pack_bf16x2(D0[s2], D1[s2]);
        }
        unsigned char* dbase = dig + (size_t)ds * DSTAGE + (isA ? 0 : S * APLANE);
        const int pstride = isA ? APLANE : BPLANE;
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2)
          *reinterpret_cast<uint4*>(dbase + (size_t)s2 * pstride + off) =
              make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
        fence_proxy_async();
        mbar_arrive(&dfull[ds]);
      }
      if (!ok) break;
    }
  } else if (warp == MMA_WARP) {
    // ======================== MMA issuer; item i uses TMEM columns from
    // (i % NBUF) NACC NT, one 64-column accumulator per digit level
    if (lane == 0) {
      const uint32_t idesc = make_idesc(128, NT);
      uint32_t g = 0, li = 0;
      for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
        const long long b = w / (2 * ntile);
        if (a.active && !a.active[b]) continue;
        const int buf = (int)(li % NBUF);
        if (!mbar_wait(&tempty[buf], ((li / NBUF) & 1) ^ 1, abort_flag, tcount)) break;
        tc_fence_after();
        uint32_t touched = 0;
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++g) {
          const int ds = (int)(g % DSTAGES);
          if (!mbar_wait(&dfull[ds], (g / DSTAGES) & 1, abort_flag, tcount)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sA = smem_u32(dig + (size_t)ds * DSTAGE);
          const uint32_t sB = sA + S * APLANE;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2) {
#pragma unroll
            for (int t = 0; t < S; ++t) {
              if (s2 + t > L) continue;
              const int acc = s2 + t;
              const uint64_t ad = tc::make_desc(sA + s2 * APLANE, 128, SBO_T);
              const uint64_t bd = tc::make_desc(sB + t * BPLANE, 128, SBO_T);
              umma(tmem + (uint32_t)((buf * NACC + acc) * NT), ad, bd, idesc,
                   (touched >> acc) & 1);
              touched |= 1u << acc;
            }
          }
          umma_commit(&dempty[ds]);
        }
        if (!ok) break;
        umma_commit(&tfull[buf]);
        ++li;
      }
      umma_commit(drain);
      int zero = 0;
      volatile int* never = &zero;
      mbar_wait(drain, 0, never, tcount);
    }
    __syncwarp();
  } else {
    // ======================== epilogue (warps 0-3 own TMEM lanes 0-127 = rows of C)
    const int row = warp * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const float alpha = (float)a.alpha_re, beta = (float)a.beta_re;
    uint32_t li = 0;
    for (long long w = blockIdx.x; w < nitems && !*abort_flag; w += gridDim.x) {
      const long long b = w / (2 * ntile);
      const int part = (int)((w / ntile) & 1), ct = (int)(w % ntile);
      if (a.active && !a.active[b]) continue;
      const int buf = (int)(li % NBUF);
      if (!mbar_wait(&tfull[buf], (li / NBUF) & 1, abort_flag, tcount)) break;
      tc_fence_after();
      const int* erow = a.scales + b * 256;
      const int* fcol = erow + 128;
      void* C = batch_ptr<double2>(a.C, b);
      const void* D = a.D.p ? batch_ptr<const double2>(a.D, b) : nullptr;
      double zpart = 0.0;
      if (a.Z.p) {
        const double2 z = *batch_ptr<const double2>(a.Z, b);
        zpart = part ? z.y : z.x;
      }
      const int ei = erow[row];
      constexpr int CW = 8;  // columns per TMEM read
#pragma unroll 1
      for (int j0 = 0; j0 < NT; j0 += CW) {
        uint32_t r[NACC][CW];
#pragma unroll
        for (int acc = 0; acc < NACC; ++acc)
          tmem_ld8(lane_base + (uint32_t)((buf * NACC + acc) * NT + j0), r[acc]);
        tmem_wait_ld();
        if (row < m) {
#pragma unroll
          for (int jj = 0; jj < CW; ++jj) {
            const int j = ct * NT + j0 + jj;
            if (j < n) {
              float hi = __uint_as_float(r[0][jj]), lo = 0.f, e;
#pragma unroll
              for (int acc = 1; acc < NACC; ++acc) {
                float s;
                two_sum(hi, __uint_as_float(r[acc][jj]), s, e);
                hi = s;
                lo += e;
              }
              float s2;
              two_sum(hi, lo, s2, e);  // normalise: |lo| <= ulp(hi)/2
              const int e2 = ei + fcol[j] - 16;
              Store<double2>::put(C, row + (long long)j * a.C.ld, part, s2, e, e2, alpha, beta,
                                  D, row + (long long)j * a.D.ld, row == j && a.Z.p, zpart);
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&tempty[buf]);
      ++li;
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == MMA_WARP) tc::tmem_dealloc(tmem, 512);
}

// 3-D tensor map (doubles, vectors or k, batch entry) of one complex128 operand
bool make_map(CUtensorMap* map, const BatchRef& R, int layout, int vecs, int K, int boxv,
              long long batch) {
  const c64t::EncodeTiled fn = c64t::encode_tiled();
  if (!fn || !R.p || R.idx || (reinterpret_cast<uintptr_t>(R.p) & 15) ||
      R.ld < (layout == MN_MAJOR ? vecs : K))
    return false;
  const cuuint64_t ldb = (cuuint64_t)R.ld * 16;
  cuuint64_t dims[3], strides[2];
  cuuint32_t box[3], es[3] = {1, 1, 1};
  if (layout == MN_MAJOR) {
    dims[0] = 2 * (cuuint64_t)vecs; dims[1] = K;
    box[0] = 2 * boxv; box[1] = KCC;
  } else {
    dims[0] = 2 * (cuuint64_t)K; dims[1] = vecs;
    box[0] = 2 * KCC; box[1] = boxv;
  }
  box[2] = 1;
  const long long entries = R.stride == 0 ? 1 : (R.mod > 0 ? R.mod : batch);
  dims[2] = (cuuint64_t)entries;
  strides[0] = ldb;
  strides[1] = R.stride == 0 ? ldb * dims[1] : (cuuint64_t)R.stride * 16;
  if (strides[1] < ldb * dims[1]) return false;  // entries must not overlap
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, R.p, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE,
            layout == K_MAJOR ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int S>
cudaError_t launch(const GemmArgs& g, cudaStream_t s, bool* used) {
  *used = false;
  Args args;
  args.g = g;
  args.layoutA = g.opA == OP_N ? MN_MAJOR : K_MAJOR;
  args.layoutB = g.opB == OP_N ? K_MAJOR : MN_MAJOR;
  alignas(64) CUtensorMap ma, mb;
  if (!make_map(&ma, g.A, args.layoutA, g.m, g.k, 128, g.batch) ||
      !make_map(&mb, g.B, args.layoutB, g.n, g.k, NT, g.batch))
    return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  constexpr int smem = Cfg<S>::SMEM;
  cudaError_t e = cudaFuncSetAttribute(zgemm_c128_tma_kernel<S>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long long gb = g.batch < 65535 ? g.batch : 65535;
  oz_scales_kernel<double2><<<dim3((unsigned)gb, 2), 256, 0, s>>>(g);
  count_launch();
  const long long items = 2LL * ((g.n + NT - 1) / NT) * g.batch;
  const int grid = (int)(items < sms ? items : sms);
  zgemm_c128_tma_kernel<S><<<grid, NTHREADS, smem, s>>>(args, ma, mb);
  count_launch();
  *used = true;
  return cudaGetLastError();
}
}  // namespace c128t

}  // namespace

cudaError_t zgemm_oz(const GemmArgs& a, int slices, int levels, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (a.m <= 0 || a.n <= 0 || a.k <= 0 || a.m > 128 || a.n > 128 || a.k > 128)
    return cudaErrorInvalidValue;
  if (a.opA == OP_T || a.opB == OP_T || a.alpha_im != 0.0 || a.beta_im != 0.0)
    return cudaErrorInvalidValue;
  (void)levels;
  if (slices == 4 || slices == 6 || slices == 7) {
    bool used = false;
    const cudaError_t e = slices == 4   ? c128t::launch<4>(a, s, &used)
                          : slices == 6 ? c128t::launch<6>(a, s, &used)
                                        : c128t::launch<7>(a, s, &used);
    if (e != cudaSuccess || used) return e;
  }
  switch (slices) {
    case 4: return launch<4, 3, 128, double2, double2>(a, s);
    case 6: return launch<6, 5, 64, double2, double2>(a, s);   // one exact accumulator per level
    case 7: return launch<7, 6, 64, double2, double2>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t zgemm_oz_c64(const GemmArgs& a, int slices, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (a.m <= 0 || a.n <= 0 || a.k <= 0 || a.m > 128 || a.n > 128 || a.k > 128)
    return cudaErrorInvalidValue;
  if (a.opA == OP_T || a.opB == OP_T || a.alpha_im != 0.0 || a.beta_im != 0.0)
    return cudaErrorInvalidValue;
  if (slices == 4) {
    bool used = false;
    const cudaError_t e = c64t::launch(a, s, &used);
    if (e != cudaSuccess || used) return e;
  }
  switch (slices) {
    case 3: return launch<3, 2, 128, float2, float2>(a, s);
    case 4: return launch<4, 3, 128, float2, float2>(a, s);
    default: return cudaErrorInvalidValue;
  }
}

int oz_timeouts_and_reset() {
  int h = 0, z = 0;
  cudaMemcpyFromSymbol(&h, g_oz_timeouts, sizeof(int));
  if (h) cudaMemcpyToSymbol(g_oz_timeouts, &z, sizeof(int));
  return h;
}

}  // namespace qt
