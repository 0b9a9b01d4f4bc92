// Host orchestration of the batched RGF sweep and the C-ABI (include/qt_rgf.h).
//
// The reference solves one (E, k) point per call of cuda_rgf_constblocksize
// (src/cuda_rgf_mod.f90:53-413), crossing the host<->device boundary around
// every cuBLAS/cuSOLVER call.  Here a WAVE of P points (P a multiple of nk,
// so point index modulo nk is the k index) advances through the sweep
// together: every block operation is one batched launch over the wave, all
// state stays in HBM, and only final reductions leave the device.
//
// Per wave:
//   1. Sancho-Rubio decimation of both leads, batched, with a per-point
//      convergence mask (src/cuda_rgf_mod.f90:657-765).
//   2. left contact   (src/cuda_rgf_mod.f90:90-134)
//   3. forward sweep  g_l, g^<_l (src/cuda_rgf_mod.f90:140-188)
//   4. right contact  G_NN, G^<_NN, tr (src/cuda_rgf_mod.f90:192-277)
//   5. backward sweep G_l, G^<_l (src/cuda_rgf_mod.f90:283-381), with the
//      7-product form (see the notes at the backward loop), and on
//      request the bond currents (:293-318)
//   6. left-contact current tre (src/cuda_rgf_mod.f90:387-407)
//   7. optional Caroli T(E) from the left-connected chain G_{N1}.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qt_rgf.h"
#include "qt_abi.h"
#include "qt_common.cuh"
#include "qt_kernels.h"

using qt::BatchRef;
using qt::cd;

namespace {
thread_local std::string g_last_error;
}

extern "C" void qt_set_last_error(const char* msg, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s (%s:%d)", msg, file, line);
  g_last_error = buf;
}

extern "C" const char* qt_last_error(void) { return g_last_error.c_str(); }

namespace {
std::atomic<long long> g_launches{0};
}
void qt::count_launch(long long n) { g_launches += n; }
extern "C" int64_t qt_kernel_launches(void) { return g_launches.load(); }
extern "C" const char* qt_version(void) { return "qtgpu 0.1 sm_103a"; }

// Optional CUDA-event timing of the block products and inverses on the
// context's stream (qt_ctx_profile): kinds 0 complex64 split product,
// 1 complex128 split product, 2 FP64 product, 3 FP32 inverse, 4 FP64 inverse;
// and of the GW map's phases: 5 the RGF of G, 6 the energy correlations and
// convolutions of P and Sigma, 7 the screened interaction W, 8 the band,
// recombination, symmetrisation and edge blocks of Sigma.  A phase's products and
// inverses are also counted in kinds 0-4.
struct Prof {
  struct Entry {
    int kind;
    cudaEvent_t a, b;
    double alg, tensor;
  };
  bool on = false;
  std::vector<Entry> v;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
};

// One timed phase on a stream while profiling is on: an event at construction, the
// closing event at end() or destruction (an early error return still closes it).
struct ProfPhase {
  Prof& p;
  cudaStream_t s;
  int kind;
  cudaEvent_t a = nullptr;
  ProfPhase(Prof& prof, cudaStream_t stream, int k) : p(prof), s(stream), kind(k) {
    if (p.on) {
      a = p.get();
      cudaEventRecord(a, s);
    }
  }
  void end() {
    if (!a) return;
    cudaEvent_t b = p.get();
    cudaEventRecord(b, s);
    p.v.push_back({kind, a, b, 0.0, 0.0});
    a = nullptr;
  }
  ~ProfPhase() { end(); }
  ProfPhase(const ProfPhase&) = delete;
  ProfPhase& operator=(const ProfPhase&) = delete;
};

struct qt_ctx {
  Prof prof;
  int device = 0;
  cudaStream_t stream = nullptr;      // where every launch of this context goes
  cudaStream_t own_stream = nullptr;  // created with the context, destroyed with it
  int64_t scratch_limit = 48LL << 30;
  int64_t wave_points = 0;  // points per wave; 0 = 4 work items per SM (608 on 152 SMs)
  void* arena = nullptr;
  size_t arena_bytes = 0;
  void* io = nullptr;  // staging for host-pointer calls
  size_t io_bytes = 0;
  void* conv = nullptr;  // complex64 copies of H / sigma for the split-precision sweep
  size_t conv_bytes = 0;
  int* fallbacks = nullptr;  // device counter: inverses redone in FP64 by the guard
  // GW k-point grid of the stage entry points (nky x nkz, 1 x 1 = one k-point) and the
  // band half-width of P and Sigma (< 0: full blocks), set by qt_ctx_set_gw_grid
  int gw_nky = 1, gw_nkz = 1, gw_ndiag = -1;
};

int qt::ctx_device(const qt_ctx* c) { return c->device; }
cudaStream_t qt::ctx_stream(const qt_ctx* c) { return c->stream; }

namespace {

constexpr double BOLTZ = 8.61734e-05;  // eV/K, src/cuda_rgf_mod.f90:22

qt_status ensure(void*& p, size_t& have, size_t need) {
  if (need <= have) return QT_OK;
  if (p) cudaFree(p);
  p = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(&p, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    QT_FAIL(QT_ERR_NOMEM, "device allocation failed");
  }
  have = need;
  return QT_OK;
}

struct Arena {
  char* base;
  size_t cap, off = 0;
  template <typename T>
  T* take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    if (off + bytes > cap) return nullptr;
    T* r = reinterpret_cast<T*>(base + off);
    off += bytes;
    return r;
  }
};

inline BatchRef ref(const void* p, long long stride, int ld, int mod = 0, const int* idx = nullptr) {
  BatchRef r;
  r.p = const_cast<void*>(p);
  r.stride = stride;
  r.mod = mod;
  r.ld = ld;
  r.idx = idx;
  return r;
}
inline BatchRef nullref() { return ref(nullptr, 0, 1); }

__global__ void make_z_kernel(const double* E, long long p0, long long P, int nk, double eta,
                              cd* z) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < P;
       b += (long long)gridDim.x * blockDim.x) {
    z[b] = cd{E[(p0 + b) / nk], eta};
  }
}

// fermi factors per point: f = 1/(1+exp((E-mu)/(k T)))  (src/cuda_rgf_mod.f90:859-863)
__global__ void make_fermi_kernel(const double* E, long long p0, long long P, int nk, double mu,
                                  double temp, double* f) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < P;
       b += (long long)gridDim.x * blockDim.x) {
    f[b] = 1.0 / (1.0 + exp((E[(p0 + b) / nk] - mu) / (BOLTZ * temp)));
  }
}

__global__ void sancho_update_kernel(long long P, const double* err, const double* err2,
                                     double tol, int it, unsigned char* active, int* iters,
                                     int* n_active) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < P;
       b += (long long)gridDim.x * blockDim.x) {
    if (!active[b]) continue;
    iters[b] = it;
    const double e = err2 ? fmax(fabs(err[b]), fabs(err2[b])) : fabs(err[b]);
    if (e < tol) active[b] = 0;
    else atomicAdd(n_active, 1);
  }
}

// status[b] |= st2[b] | st2[P + b]: both leads' decimation flags of point b
__global__ void or_halves_kernel(long long P, const int* st2, int* status) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < P;
       b += (long long)gridDim.x * blockDim.x)
    status[b] |= st2[b] | st2[P + b];
}

__global__ void flag_unconverged_kernel(long long P, const unsigned char* active, int* status) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < P;
       b += (long long)gridDim.x * blockDim.x)
    if (active[b]) status[b] |= qt::PT_SANCHO_NOT_CONVERGED;
}

// status[b] |= NONFINITE when any of the `row` doubles of point b's output is NaN/Inf
// (one warp per point; the outputs are what the caller reads)
__global__ void check_outputs_kernel(long long P, long long row, const double* data, int* status) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long b = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; b < P; b += warps) {
    bool bad = false;
    for (long long i = lane; i < row; i += 32) bad |= !isfinite(data[b * row + i]);
    if (__any_sync(0xffffffffu, bad) && lane == 0) status[b] |= qt::PT_NONFINITE;
  }
}

inline unsigned g1d(long long n) {
  long long g = (n + 255) / 256;
  if (g < 1) g = 1;
  if (g > 65535LL * 8) g = 65535LL * 8;
  return (unsigned)g;
}

__global__ void flat_d2f_kernel(const double2* x, float2* y, long long count) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x)
    y[t] = make_float2((float)x[t].x, (float)x[t].y);
}

// ----------------------------------------------------------------- ops
// Block operations on storage TC.  Plain path: TC = double2 on the FP64
// pipes.  Split path: TC = double2 with FP64-grade digits (Sancho and the
// contact self-energies) or TC = float2 with `slices` digits (the sweep);
// inverses are FP32 eliminations followed by `refine` residual steps
// X <- X + X (I - A X) computed with the tensor-core product.
// The split path's kernels take one 128-row tile.  Larger blocks (up to
// MAX_SPLIT = 384 orbitals) are tiled here: products over near-equal tiles of
// <= 128, inverses by the 2 x 2 block form over such tiles.
constexpr int SPLIT_TILE = 128;
constexpr int MAX_SPLIT = 3 * SPLIT_TILE;

template <typename TC>
struct Ops {
  cudaStream_t s;
  int n;
  qt_precision prec;
  int slices = 4;
  int refine = 1;
  const cd* one = nullptr;  // device scalar (1, 0)
  Prof* prof = nullptr;     // optional launch timing
  int* scales = nullptr;    // P * 256 ints: exponent scratch of the split product
  TC* rt1 = nullptr;        // P * n*n refinement scratch
  TC* rt2 = nullptr;
  long long P = 0;
  // Inverse guard (split path): entries whose first residual R = I - A X is too large for
  // the refinement to converge safely get an FP64 elimination instead.  guard: P flags;
  // fbw: P * n*n complex128 workspace (complex64 storage only); fallbacks: count.
  unsigned char* guard = nullptr;
  cd* fbw = nullptr;
  int* fallbacks = nullptr;
  double guard_tol() const {
    // refinement diverges once ||R||_2 >= 1, and ||R||_F >= ||R||_2: with several steps
    // to follow, 0.25 leaves margin; a single step (the complex64 sweep) only needs the
    // divergent entries redone.  QT_GUARD_TOL overrides for accuracy studies.
    const char* v = getenv("QT_GUARD_TOL");
    if (v && *v) return atof(v);
    return refine > 1 ? 0.25 : 1.0;
  }

  qt_status gemm(BatchRef A, int opA, BatchRef B, int opB, BatchRef C, long long batch,
                 cd alpha = {1, 0}, BatchRef D = nullref(), cd beta = {0, 0},
                 BatchRef Z = nullref(), const unsigned char* active = nullptr) {
    return gemm3(n, n, n, A, opA, B, opB, C, batch, alpha, D, beta, Z, active);
  }
  // part t of x split into nt near-equal parts: offset and length
  static void part(int x, int nt, int t, int& off, int& len) {
    const int base = x / nt, rem = x % nt;
    off = t * base + (t < rem ? t : rem);
    len = base + (t < rem ? 1 : 0);
  }
  // the sub-block of R starting at row r, column c (same batch addressing)
  static BatchRef sub(BatchRef R, int r, int c) {
    if (R.p)
      R.p = static_cast<char*>(R.p) + ((long long)r + (long long)c * R.ld) * (long long)sizeof(TC);
    return R;
  }
  // C (m x nn) = alpha op(A) op(B) + beta D + z I, op(A) m x k, op(B) k x nn.  On the split
  // path, sizes above one tile are tiled: every C tile accumulates its K tiles in place (the
  // product's epilogue reads D and writes C element by element in the same thread), and
  // z I goes to the diagonal tiles (m == nn, so rows and columns are tiled alike).
  qt_status gemm3(int m, int nn, int k, BatchRef A, int opA, BatchRef B, int opB, BatchRef C,
                  long long batch, cd alpha = {1, 0}, BatchRef D = nullref(), cd beta = {0, 0},
                  BatchRef Z = nullref(), const unsigned char* active = nullptr,
                  int digits = 0) {
    if (prec == QT_PREC_FP64 || (m <= SPLIT_TILE && nn <= SPLIT_TILE && k <= SPLIT_TILE))
      return gemm3_one(m, nn, k, A, opA, B, opB, C, batch, alpha, D, beta, Z, active, digits);
    if (m > MAX_SPLIT || nn > MAX_SPLIT || k > MAX_SPLIT)
      QT_FAIL(QT_ERR_UNSUPPORTED, "split product: blocks above the tiling limit");
    const int mt = (m + SPLIT_TILE - 1) / SPLIT_TILE, nt = (nn + SPLIT_TILE - 1) / SPLIT_TILE;
    const int kt = (k + SPLIT_TILE - 1) / SPLIT_TILE;
    for (int i = 0; i < mt; ++i)
      for (int j = 0; j < nt; ++j) {
        int r0, rl, c0, cl;
        part(m, mt, i, r0, rl);
        part(nn, nt, j, c0, cl);
        const BatchRef Ct = sub(C, r0, c0);
        for (int t = 0; t < kt; ++t) {
          int k0, kl;
          part(k, kt, t, k0, kl);
          const BatchRef At = opA == qt::OP_N ? sub(A, r0, k0) : sub(A, k0, r0);
          const BatchRef Bt = opB == qt::OP_N ? sub(B, k0, c0) : sub(B, c0, k0);
          const bool first = t == 0;
          const BatchRef Dt = first ? (D.p ? sub(D, r0, c0) : nullref()) : Ct;
          const BatchRef Zt = (first && Z.p && m == nn && i == j) ? Z : nullref();
          QT_TRY(gemm3_one(rl, cl, kl, At, opA, Bt, opB, Ct, batch, alpha, Dt,
                           first ? beta : cd{1, 0}, Zt, active, digits));
        }
      }
    return QT_OK;
  }
  // one kernel launch: every size <= 128 on the split path
  qt_status gemm3_one(int m, int nn, int k, BatchRef A, int opA, BatchRef B, int opB, BatchRef C,
                      long long batch, cd alpha, BatchRef D, cd beta, BatchRef Z,
                      const unsigned char* active, int digits) {
    const int sl = digits ? digits : slices;
    qt::GemmArgs g;
    g.m = m;
    g.n = nn;
    g.k = k;
    g.A = A; g.B = B; g.C = C; g.D = D; g.Z = Z;
    g.opA = opA; g.opB = opB;
    g.alpha_re = alpha.x; g.alpha_im = alpha.y; g.beta_re = beta.x; g.beta_im = beta.y;
    g.batch = batch;
    g.active = active;
    g.scales = scales;
    if (prec != QT_PREC_FP64 && (!scales || batch > P)) QT_FAIL(QT_ERR_ARG, "split product scratch too small");
    cudaError_t e;
    const bool timed = prof && prof->on;
    cudaEvent_t ea = nullptr, eb = nullptr;
    if (timed) { ea = prof->get(); eb = prof->get(); cudaEventRecord(ea, s); }
    int kind;
    if constexpr (sizeof(TC) == 16) {
      kind = prec == QT_PREC_FP64 ? 2 : 1;
      e = prec == QT_PREC_FP64 ? qt::zgemm_f64(g, s) : qt::zgemm_oz(g, sl, sl - 1, s);
    } else {
      kind = 0;
      e = qt::zgemm_oz_c64(g, sl, s);
    }
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    if (timed) {
      cudaEventRecord(eb, s);
      // algorithmic: 8 m n k real flops per complex block product; executed on the tensor
      // pipe: 2 real parts x digit pairs x 2 x 128 x npad x K'
      const double alg = 8.0 * m * (double)nn * k * batch;
      double tens = 0.0;
      if (kind != 2) {
        const int L = sl - 1, npad = (nn + 15) / 16 * 16, kp = (k + 15) / 16 * 16;
        int pairs = 0;
        for (int a = 0; a < sl; ++a)
          for (int b = 0; b < sl; ++b) pairs += (a + b <= L);
        tens = 2.0 * pairs * 2.0 * 128.0 * npad * (2.0 * kp) * batch;
      }
      prof->v.push_back({kind, ea, eb, alg, tens});
    }
    return QT_OK;
  }
  // X = inv(A); A is preserved (X must differ from A in the split path)
  qt_status inv(BatchRef A, BatchRef X, long long batch, int* status,
                const unsigned char* active = nullptr, int nn = 0) {
    if (nn <= 0) nn = n;
    qt::InvArgs a;
    a.n = nn; a.A = A; a.X = X; a.batch = batch; a.status = status; a.active = active;
    cudaError_t e;
    const bool timed = prof && prof->on;
    cudaEvent_t ea = nullptr, eb = nullptr;
    if (timed) { ea = prof->get(); eb = prof->get(); cudaEventRecord(ea, s); }
    const double alg = 8.0 * nn * (double)nn * nn * batch;  // inversion counted as one n^3 product
    if (prec == QT_PREC_FP64) {
      if constexpr (sizeof(TC) == 16) e = qt::zinv_f64(a, s);
      else e = cudaErrorInvalidValue;
      if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      if (timed) { cudaEventRecord(eb, s); prof->v.push_back({4, ea, eb, alg, 0.0}); }
      return QT_OK;
    }
    if (X.p == A.p) QT_FAIL(QT_ERR_ARG, "split-precision inverse needs X != A");
    if (refine > 0 && (batch > P || !rt1 || !rt2)) QT_FAIL(QT_ERR_ARG, "refinement scratch too small");
    if (nn <= SPLIT_TILE) {
      e = qt::zinv_f32<TC>(a, s);
      if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      if (timed) { cudaEventRecord(eb, s); prof->v.push_back({3, ea, eb, alg, 0.0}); }
    } else {
      if (timed) { cudaEventDestroy(ea); cudaEventDestroy(eb); }
      QT_TRY(inv_blocks(A, X, nn, batch, status, active));
    }
    // refinement scratch holds batch blocks of the widest size (stride n*n).  Only the
    // residual R = I - A X needs the full digits; the update X R is |R| times smaller than X,
    // so 4 digits (2^-28 of |X||R|) leave X's accuracy to R's.
    const BatchRef R = ref(rt1, (long long)n * n, nn), T = ref(rt2, (long long)n * n, nn);
    const bool guarded = guard && (sizeof(TC) == 16 || fbw);
    if (guarded && batch > P) QT_FAIL(QT_ERR_ARG, "inverse guard scratch too small");
    // With three or more steps on one-tile blocks, the last step runs only for entries whose
    // previous residual has ||R||_F > 3e-9: R_{k+1} = R_k^2 up to the products' rounding, so
    // the others are at FP64 resolution already (||R|| <= 1e-17).  The guard flags hold that
    // mask once the FP64 redo of step 0 has read them.  Blocks above one tile start from the
    // 2 x 2 block form, where the last step was measured to still pay (a 4.5x larger T(E)
    // error without it on an ill-conditioned device), so they keep every step.
    const bool skip_last = guarded && refine >= 3 && nn <= SPLIT_TILE && !getenv("QT_REFINE_ALL");
    for (int it = 0; it < refine; ++it) {
      const bool masked = skip_last && it == refine - 1;
      const unsigned char* act = masked ? guard : active;
      QT_TRY(gemm3(nn, nn, nn, A, qt::OP_N, X, qt::OP_N, R, batch, cd{-1, 0}, nullref(),
                   cd{0, 0}, ref(one, 0, 1), act));  // R = I - A X
      if (it == 0 && guarded) {
        e = qt::zinv_guard<TC>(nn, batch, R, active, guard_tol(), guard, fallbacks, s);
        if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      }
      if (skip_last && it == refine - 2) {
        e = qt::zinv_guard<TC>(nn, batch, R, active, 3e-9, guard, nullptr, s);
        if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      }
      QT_TRY(gemm3(nn, nn, nn, X, qt::OP_N, R, qt::OP_N, T, batch, cd{1, 0}, X, cd{1, 0},
                   nullref(), act, 4));
      if (masked) {
        e = qt::zaxpby<TC>(nn, batch, T, 1.0, 0.0, nullref(), 0.0, 0.0, nullref(), X, act, s);
        if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      } else {
        qt::zcopy<TC>(nn, batch, T, X, s);
      }
      if (it == 0 && guarded) {  // flagged entries: FP64 elimination from A
        qt::InvArgs f;
        f.n = nn; f.A = A; f.X = X; f.batch = batch; f.status = status; f.active = guard;
        e = qt::zinv_f64_ws<TC>(f, fbw, (long long)n * n, s);
        if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      }
    }
    return QT_OK;
  }
  // X = inv(A) for nn > 128 on the split path, without refinement: with
  // A = [P Q; R S], P p x p, S s x s (s = nn/2 up to 256, else 128, so S is one tile),
  //   X11 = P^-1 (recursing while p > 128), T = R X11, Sc = S - T Q, X22 = Sc^-1,
  //   U = X11 Q, X12 = -U X22, X21 = -X22 T, X11 <- X11 - X12 T.
  // T and U sit in rt1, Sc in rt2 (each holds n*n per entry); the recursion on P runs
  // before either is in use.  Singular tiles set the entry's status bits.
  qt_status inv_blocks(BatchRef A, BatchRef X, int nn, long long batch, int* status,
                       const unsigned char* active) {
    if (nn > MAX_SPLIT) QT_FAIL(QT_ERR_UNSUPPORTED, "split inverse: block above the tiling limit");
    if (!rt1 || !rt2 || batch > P) QT_FAIL(QT_ERR_ARG, "block-inverse scratch too small");
    const int s_ = nn > 2 * SPLIT_TILE ? SPLIT_TILE : nn / 2, p = nn - s_;
    const BatchRef Q = sub(A, 0, p), R = sub(A, p, 0), S = sub(A, p, p);
    const BatchRef X11 = X, X12 = sub(X, 0, p), X21 = sub(X, p, 0), X22 = sub(X, p, p);
    if (p > SPLIT_TILE) {
      QT_TRY(inv_blocks(A, X11, p, batch, status, active));
    } else {
      qt::InvArgs a;
      a.n = p; a.A = A; a.X = X11; a.batch = batch; a.status = status; a.active = active;
      cudaError_t e = qt::zinv_f32<TC>(a, s);
      if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    }
    const long long st = (long long)n * n;
    const BatchRef T = ref(rt1, st, s_);                  // s x p
    const BatchRef U = ref(rt1 + (size_t)s_ * p, st, p);  // p x s
    const BatchRef Sc = ref(rt2, st, s_);                 // s x s
    QT_TRY(gemm3(s_, p, p, R, qt::OP_N, X11, qt::OP_N, T, batch, cd{1, 0}, nullref(), cd{0, 0},
                 nullref(), active));
    QT_TRY(gemm3(s_, s_, p, T, qt::OP_N, Q, qt::OP_N, Sc, batch, cd{-1, 0}, S, cd{1, 0},
                 nullref(), active));
    {
      qt::InvArgs a;
      a.n = s_; a.A = Sc; a.X = X22; a.batch = batch; a.status = status; a.active = active;
      cudaError_t e = qt::zinv_f32<TC>(a, s);
      if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    }
    QT_TRY(gemm3(p, s_, p, X11, qt::OP_N, Q, qt::OP_N, U, batch, cd{1, 0}, nullref(), cd{0, 0},
                 nullref(), active));
    QT_TRY(gemm3(p, s_, s_, U, qt::OP_N, X22, qt::OP_N, X12, batch, cd{-1, 0}, nullref(),
                 cd{0, 0}, nullref(), active));
    QT_TRY(gemm3(s_, p, s_, X22, qt::OP_N, T, qt::OP_N, X21, batch, cd{-1, 0}, nullref(),
                 cd{0, 0}, nullref(), active));
    QT_TRY(gemm3(p, p, s_, X12, qt::OP_N, T, qt::OP_N, X11, batch, cd{-1, 0}, X11, cd{1, 0},
                 nullref(), active));
    return QT_OK;
  }
};

// ----------------------------------------------------------- the solve
struct Problem {
  int nm, nx, nk;
  long long npts;
  const cd* Hii; long long hk, hl;   // complex128 blocks (device)
  const cd* H1i; long long h1k, h1l;
  const float2* Hii32;               // complex64 copies (split path)
  const float2* H1i32;
  const cd* sigr;                    // per point [npts][nx][nm2] or null
  const cd* sigl;
  const float2* sigr32;
  const float2* sigl32;
  const double* E;
  qt_contacts c;
  qt_precision prec;
  unsigned flags;
  int sweep_slices, lead_slices;
  int sweep_refine;  // refinement steps of the sweep's FP32 inverses (split paths)
  // device outputs (may be null)
  double *tr, *tre, *T, *dgr, *dgl, *dgg;
  cd *Gr, *Gl, *Gg;
  double* bond;  // [npts][nx-1] bond currents
  cd* Jd;        // [npts][nx][nm2] bond-current blocks
  int *status, *iters;
};

size_t wave_bytes(const Problem& pb, long long P) {
  const size_t nm2 = (size_t)pb.nm * pb.nm;
  const size_t tc = pb.prec == QT_PREC_MIXED ? 8 : 16;  // complex64 sweep only in MIXED
  const size_t sweep = (2 * (size_t)pb.nx + 14 + 2) * tc;  // g_l, g^<_l, temporaries, refinement
  const size_t lead = (2 * (7 + 2) + 6) * 16;  // Sancho state + refinement of both leads + contact
  const size_t guard = tc == 8 ? 16 : 0;        // complex128 workspace of the inverse guard
  return (sweep + lead + guard) * nm2 * P + (size_t)P * 4096 + (512 << 10);
}

// Batched Sancho-Rubio on the wave (complex128 state).  H00 per point, H_10 the
// decimation's coupling argument (dag_in: it is H10in^+, the left lead,
// src/cuda_rgf_mod.f90:101).  G00 = (zS - H_SS)^-1, GBB = (zS - H_BB)^-1.
//
// With G00b set, the same run also yields the surface Green's function of the chain
// that extends the other way (the dual surface): H_S'S' accumulates H_10 A H_01, the
// term H_BB already receives, and the run stops when both couplings are below tol.  A
// lead pair that is one chain (equal on-site blocks and couplings, the right lead
// called with H10 where the left is called with H10^+) costs one decimation, not two.
qt_status sancho_wave(const Ops<double2>& op0, Arena& ar, long long P, BatchRef H00,
                      BatchRef H10in, bool dag_in, const cd* zlead, double tol, int max_iter,
                      BatchRef G00, BatchRef GBB, int* status, int* iters_out, int iters_stride,
                      BatchRef G00b = nullref(), bool reset_on_max = false) {
  Ops<double2> op = op0;
  const int n = op.n;
  const long long nm2 = (long long)n * n;
  cudaStream_t s = op.s;
  const size_t mark = ar.off;  // the Sancho state is released on return
  const bool dual = G00b.p != nullptr;
  cd* buf = ar.take<cd>((size_t)(dual ? 8 : 7) * P * nm2);
  double* err = ar.take<double>(P);
  double* err2 = dual ? ar.take<double>(P) : nullptr;
  unsigned char* active = ar.take<unsigned char>(P);
  int* iters = ar.take<int>(P);
  int* nact = ar.take<int>(1);
  if (op.prec != QT_PREC_FP64) {
    op.rt1 = reinterpret_cast<double2*>(ar.take<cd>((size_t)P * nm2));
    op.rt2 = reinterpret_cast<double2*>(ar.take<cd>((size_t)P * nm2));
    if (!op.scales || op.P < P) op.scales = ar.take<int>((size_t)P * 256);
    op.P = P;
    if (!op.rt1 || !op.rt2) QT_FAIL(QT_ERR_NOMEM, "wave arena exhausted (sancho refinement)");
  }
  if (!buf || !err || !active || !iters || !nact || (dual && !err2))
    QT_FAIL(QT_ERR_NOMEM, "wave arena exhausted (sancho)");
  BatchRef HBB = ref(buf + 0 * P * nm2, nm2, n), HSS = ref(buf + 1 * P * nm2, nm2, n);
  BatchRef H10 = ref(buf + 2 * P * nm2, nm2, n), H01 = ref(buf + 3 * P * nm2, nm2, n);
  BatchRef A = ref(buf + 4 * P * nm2, nm2, n), B = ref(buf + 5 * P * nm2, nm2, n);
  BatchRef C = ref(buf + 6 * P * nm2, nm2, n);
  const BatchRef HSS2 = dual ? ref(buf + 7 * P * nm2, nm2, n) : nullref();
  const BatchRef Zl = ref(zlead, 1, 1);
  qt::zcopy<double2>(n, P, H00, HBB, s);
  qt::zcopy<double2>(n, P, H00, HSS, s);
  if (dual) qt::zcopy<double2>(n, P, H00, HSS2, s);
  if (dag_in) {
    qt::zdagger<double2>(n, P, H10in, H10, s);
    qt::zcopy<double2>(n, P, H10in, H01, s);
  } else {
    qt::zcopy<double2>(n, P, H10in, H10, s);
    qt::zdagger<double2>(n, P, H10in, H01, s);
  }
  cudaMemsetAsync(active, 1, P, s);
  cudaMemsetAsync(iters, 0, P * sizeof(int), s);
  const cd one{1, 0};
  for (int it = 1; it <= max_iter; ++it) {
    // A = (z S - H_BB)^-1           (src/cuda_rgf_mod.f90:687-696)
    qt::zaxpby<double2>(n, P, HBB, -1, 0, nullref(), 0, 0, Zl, C, active, s);
    QT_TRY(op.inv(C, A, P, status, active));
    // B = A H_10 ; H_SS += H_01 B ; H_BB += H_01 B      (:698-702)
    QT_TRY(op.gemm(A, qt::OP_N, H10, qt::OP_N, B, P, one, nullref(), {0, 0}, nullref(), active));
    QT_TRY(op.gemm(H01, qt::OP_N, B, qt::OP_N, C, P, one, nullref(), {0, 0}, nullref(), active));
    qt::zadd2<double2>(n, P, C, HSS, HBB, active, s);  // H_SS += C ; H_BB += C
    // C = H_10 B ; B = A H_01 ; A = H_10 B ; H_10 = C ; H_BB += A    (:704-711)
    QT_TRY(op.gemm(H10, qt::OP_N, B, qt::OP_N, C, P, one, nullref(), {0, 0}, nullref(), active));
    QT_TRY(op.gemm(A, qt::OP_N, H01, qt::OP_N, B, P, one, nullref(), {0, 0}, nullref(), active));
    QT_TRY(op.gemm(H10, qt::OP_N, B, qt::OP_N, A, P, one, nullref(), {0, 0}, nullref(), active));
    std::swap(H10, C);
    if (dual) qt::zadd2<double2>(n, P, A, HBB, HSS2, active, s);  // H_BB += A ; H_SS2 += A
    else qt::zaxpby<double2>(n, P, HBB, 1, 0, A, 1, 0, nullref(), HBB, active, s);
    // H_01 = H_01 B ; error = sum |H_01|            (:712-726)
    QT_TRY(op.gemm(H01, qt::OP_N, B, qt::OP_N, C, P, one, nullref(), {0, 0}, nullref(), active));
    std::swap(H01, C);
    qt::zabssum<double2>(n, P, H01, err, active, tol, s);
    if (dual) qt::zabssum<double2>(n, P, H10, err2, active, tol, s);  // the dual run's H_01
    cudaMemsetAsync(nact, 0, sizeof(int), s);
    sancho_update_kernel<<<g1d(P), 256, 0, s>>>(P, err, err2, tol, it, active, iters, nact);
    qt::count_launch();
    if ((it % 4) == 0 || it == max_iter) {
      int h = 0;
      cudaMemcpyAsync(&h, nact, sizeof(int), cudaMemcpyDeviceToHost, s);
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
      if (h == 0) break;
    }
  }
  if (reset_on_max) {
    // green_RGF_RS's decimation (src/gw_mod.f90:1440-1445): an entry still unconverged after
    // max_iter steps restarts from H_SS = H_BB = H00, i.e. G00 = GBB = (z S - H00)^-1
    for (const BatchRef& Hx : {HSS, HBB, HSS2})
      if (Hx.p) qt::zaxpby<double2>(n, P, H00, 1, 0, nullref(), 0, 0, nullref(), Hx, active, s);
  }
  flag_unconverged_kernel<<<g1d(P), 256, 0, s>>>(P, active, status);
  qt::count_launch();
  // G00 = (z S - H_SS)^-1 ; GBB = (z S - H_BB)^-1    (:740-761)
  qt::zaxpby<double2>(n, P, HSS, -1, 0, nullref(), 0, 0, Zl, C, nullptr, s);
  QT_TRY(op.inv(C, G00, P, status));
  if (dual) {
    qt::zaxpby<double2>(n, P, HSS2, -1, 0, nullref(), 0, 0, Zl, C, nullptr, s);
    QT_TRY(op.inv(C, G00b, P, status));
  }
  if (GBB.p) {
    qt::zaxpby<double2>(n, P, HBB, -1, 0, nullref(), 0, 0, Zl, C, nullptr, s);
    QT_TRY(op.inv(C, GBB, P, status));
  }
  if (iters_out)
    cudaMemcpy2DAsync(iters_out, iters_stride * sizeof(int), iters, sizeof(int), sizeof(int), P,
                      cudaMemcpyDeviceToDevice, s);
  ar.off = mark;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

// non-finite outputs of a wave: diagonals (diag complex values per point) and traces
void check_wave_outputs(long long P, long long diag, long long p0, const double* dgr,
                        const double* dgl, const double* dgg, const double* T, const double* tr,
                        const double* tre, int* status, cudaStream_t s) {
  const unsigned grid = (unsigned)std::min<long long>((P + 7) / 8, 4096);
  for (const double* d : {dgr, dgl, dgg})
    if (d) {
      check_outputs_kernel<<<grid, 256, 0, s>>>(P, 2 * diag, d + 2 * p0 * diag, status);
      qt::count_launch();
    }
  for (const double* d : {T, tr, tre})
    if (d) {
      check_outputs_kernel<<<grid, 256, 0, s>>>(P, 1, d + p0, status);
      qt::count_launch();
    }
}

template <typename TC>
void zconvert_or_copy(int n, long long P, BatchRef X, BatchRef Y, cudaStream_t s) {
  if constexpr (sizeof(TC) == 16) qt::zcopy<double2>(n, P, X, Y, s);
  else qt::zconvert<double2, float2>(n, P, X, Y, s);
}
template <typename TC>
void to_c128(int n, long long P, BatchRef X, BatchRef Y, cudaStream_t s) {
  if constexpr (sizeof(TC) == 16) qt::zcopy<double2>(n, P, X, Y, s);
  else qt::zconvert<float2, double2>(n, P, X, Y, s);
}

template <typename TC>
qt_status solve_wave(qt_ctx* ctx, const Problem& pb, long long p0, long long P, Arena& ar) {
  const int n = pb.nm, nx = pb.nx, nk = pb.nk;
  const long long nm2 = (long long)n * n;
  cudaStream_t s = ctx->stream;
  const unsigned q = pb.c.quirks;
  const bool split = pb.prec != QT_PREC_FP64;

  cd* zint = ar.take<cd>(P);
  cd* zlead = ar.take<cd>(P);
  double* fl = ar.take<double>(P);
  double* fr = ar.take<double>(P);
  double* fe = ar.take<double>(P);
  cd* one = ar.take<cd>(1);
  int* status = ar.take<int>(P);
  TC* gl_all = ar.take<TC>((size_t)nx * P * nm2);   // g_l   [l][b]
  TC* gln_all = ar.take<TC>((size_t)nx * P * nm2);  // g^<_l [l][b]
  TC* tmp = ar.take<TC>((size_t)14 * P * nm2);
  TC* rt1 = ar.take<TC>((size_t)P * nm2);
  TC* rt2 = ar.take<TC>((size_t)P * nm2);
  cd* cbuf = ar.take<cd>((size_t)6 * P * nm2);      // complex128 contact scratch
  int* scales = ar.take<int>((size_t)P * 256);       // split-product exponent scratch
  unsigned char* guard = ar.take<unsigned char>((size_t)2 * P);  // both leads' 2P entries
  cd* fbw = sizeof(TC) == 8 ? ar.take<cd>((size_t)P * nm2) : nullptr;
  if (!zint || !zlead || !fl || !fr || !fe || !one || !status || !gl_all || !gln_all || !tmp ||
      !rt1 || !rt2 || !cbuf || !scales || !guard || (sizeof(TC) == 8 && !fbw))
    QT_FAIL(QT_ERR_NOMEM, "wave arena exhausted");
  // sweep operations on TC, contact operations on complex128
  Ops<TC> op{s, n, pb.prec};
  op.slices = pb.sweep_slices;
  op.refine = split ? pb.sweep_refine : 0;
  op.one = one; op.rt1 = rt1; op.rt2 = rt2; op.P = P; op.scales = scales;
  op.prof = &ctx->prof;
  op.guard = guard; op.fbw = fbw; op.fallbacks = ctx->fallbacks;
  Ops<double2> cop{s, n, pb.prec};
  cop.prof = &ctx->prof;
  cop.slices = pb.lead_slices;
  cop.refine = split ? 3 : 0;  // FP32 elimination: (kappa 2^-24)^(r+1), kappa ~ 1e5 at lead band edges
  cop.one = one;
  cop.scales = scales;
  cop.P = P;
  cop.guard = guard; cop.fallbacks = ctx->fallbacks;

  const cd h1{1.0, 0.0};
  cudaMemcpyAsync(one, &h1, sizeof(cd), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(status, 0, P * sizeof(int), s);
  make_z_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, pb.c.eta_interior, zint);
  qt::count_launch();
  make_z_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, pb.c.eta_lead, zlead);
  qt::count_launch();
  // Contact Fermi pairings: GPU routine src/cuda_rgf_mod.f90:113 (mul,TEMPl), :242 (mur,TEMPl),
  // :388 (mul,TEMPr); CPU routine src/rgf_mod.f90:100 (mur,TEMPr), :182 (mul,TEMPl), :258 (mur,TEMPr).
  const bool cpu = (q & QT_QUIRK_CPU_FERMI) != 0;
  make_fermi_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, cpu ? pb.c.mur : pb.c.mul,
                                           cpu ? pb.c.tempr : pb.c.templ, fl);
  qt::count_launch();
  make_fermi_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, cpu ? pb.c.mul : pb.c.mur, pb.c.templ,
                                           fr);
  qt::count_launch();
  make_fermi_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, cpu ? pb.c.mur : pb.c.mul, pb.c.tempr,
                                           fe);
  qt::count_launch();
  const double tr_sign = cpu ? 1.0 : -1.0;

  const bool c64 = sizeof(TC) == 8;
  auto T = [&](int i) { return ref(tmp + (size_t)i * P * nm2, nm2, n); };
  auto C8 = [&](int i) { return ref(cbuf + (size_t)i * P * nm2, nm2, n); };
  auto GL = [&](int l) { return ref(gl_all + (size_t)l * P * nm2, nm2, n); };
  auto GLN = [&](int l) { return ref(gln_all + (size_t)l * P * nm2, nm2, n); };
  // Hamiltonian blocks in complex128 (contacts) and in the sweep's storage
  auto HII8 = [&](int l) { return ref(pb.Hii + l * pb.hl, pb.hk, n, pb.hk ? nk : 0); };
  auto H1I8 = [&](int l) { return ref(pb.H1i + l * pb.h1l, pb.h1k, n, pb.h1k ? nk : 0); };
  auto HII = [&](int l) {
    return c64 ? ref(pb.Hii32 + l * pb.hl, pb.hk, n, pb.hk ? nk : 0) : HII8(l);
  };
  auto H1I = [&](int l) {
    return c64 ? ref(pb.H1i32 + l * pb.h1l, pb.h1k, n, pb.h1k ? nk : 0) : H1I8(l);
  };
  auto SIGR8 = [&](int l) {
    return pb.sigr ? ref(pb.sigr + (p0 * nx + l) * nm2, nx * nm2, n) : nullref();
  };
  auto SIGR = [&](int l) {
    if (!pb.sigr) return nullref();
    return c64 ? ref(pb.sigr32 + (p0 * nx + l) * nm2, nx * nm2, n) : SIGR8(l);
  };
  auto SIGL = [&](int l) {
    if (!pb.sigl) return nullref();
    return c64 ? ref(pb.sigl32 + (p0 * nx + l) * nm2, nx * nm2, n)
               : ref(pb.sigl + (p0 * nx + l) * nm2, nx * nm2, n);
  };
  auto OUTB = [&](cd* base, int l) { return ref(base + (p0 * nx + l) * nm2, nx * nm2, n); };
  const BatchRef Zi = ref(zint, 1, 1);
  const cd one_c{1, 0}, mone{-1, 0};
  const BatchRef SigL = T(13);
  BatchRef Pch = T(12), Pnext = T(11);  // Caroli chain P_l, ping-pong
  const bool caroli = (pb.flags & QT_FLAG_CAROLI) && pb.T;

  // ---------------- both leads' decimations as one batched wave of 2P entries:
  // [0, P) the left lead, called with H10^+ (src/cuda_rgf_mod.f90:90-134), and
  // [P, 2P) the right lead (:192-277); surface Green's functions into C8(4), C8(5)
  const int N = nx - 1;
  // both leads are one chain when every slab shares H_ii and H1i and no scattering
  // self-energy touches them: one decimation gives both surfaces
  const bool reset = (q & QT_QUIRK_GW_SANCHO_RESET) != 0;
  const bool one_chain = pb.hl == 0 && pb.h1l == 0 && !pb.sigr && !reset;
  if (one_chain) {
    const size_t mark = ar.off;
    qt::zcopy<double2>(n, P, HII8(0), C8(0), s);
    qt::zdagger<double2>(n, P, H1I8(0), C8(2), s);
    int* it1 = ar.take<int>(P);
    if (!it1) QT_FAIL(QT_ERR_NOMEM, "wave arena exhausted (leads)");
    QT_TRY(sancho_wave(cop, ar, P, C8(0), C8(2), false, zlead, pb.c.sancho_tol,
                       pb.c.sancho_max_iter, C8(4), nullref(), status, it1, 1, C8(5)));
    if (pb.iters) {
      cudaMemcpy2DAsync(pb.iters + p0 * 2, 2 * sizeof(int), it1, sizeof(int), sizeof(int), P,
                        cudaMemcpyDeviceToDevice, s);
      cudaMemcpy2DAsync(pb.iters + p0 * 2 + 1, 2 * sizeof(int), it1, sizeof(int), sizeof(int),
                        P, cudaMemcpyDeviceToDevice, s);
    }
    ar.off = mark;
  } else {
    const size_t mark = ar.off;
    cd* z2 = ar.take<cd>(2 * P);
    int* st2 = ar.take<int>(2 * P);
    int* it2 = ar.take<int>(2 * P);
    if (!z2 || !st2 || !it2) QT_FAIL(QT_ERR_NOMEM, "wave arena exhausted (leads)");
    cudaMemcpyAsync(z2, zlead, P * sizeof(cd), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(z2 + P, zlead, P * sizeof(cd), cudaMemcpyDeviceToDevice, s);
    cudaMemsetAsync(st2, 0, 2 * P * sizeof(int), s);
    qt::zaxpby<double2>(n, P, HII8(0), 1, 0, SIGR8(0), 1, 0, nullref(), C8(0), nullptr, s);
    qt::zaxpby<double2>(n, P, HII8(N), 1, 0, SIGR8(N), 1, 0, nullref(), C8(1), nullptr, s);
    qt::zdagger<double2>(n, P, H1I8(0), C8(2), s);
    qt::zcopy<double2>(n, P, H1I8(N), C8(3), s);
    QT_TRY(sancho_wave(cop, ar, 2 * P, C8(0), C8(2), false, z2, pb.c.sancho_tol,
                       pb.c.sancho_max_iter, C8(4), nullref(), st2, it2, 1, nullref(), reset));
    or_halves_kernel<<<g1d(P), 256, 0, s>>>(P, st2, status);
    qt::count_launch();
    if (pb.iters) {
      cudaMemcpy2DAsync(pb.iters + p0 * 2, 2 * sizeof(int), it2, sizeof(int), sizeof(int), P,
                        cudaMemcpyDeviceToDevice, s);
      cudaMemcpy2DAsync(pb.iters + p0 * 2 + 1, 2 * sizeof(int), it2 + P, sizeof(int),
                        sizeof(int), P, cudaMemcpyDeviceToDevice, s);
    }
    ar.off = mark;
  }

  // ---------------- left contact (src/cuda_rgf_mod.f90:90-134)
  // Sigma_L = H10 G00 H10^+ at FP64 grade, then stored as TC
  QT_TRY(cop.gemm(H1I8(0), qt::OP_N, C8(4), qt::OP_N, C8(2), P));
  QT_TRY(cop.gemm(C8(2), qt::OP_N, H1I8(0), qt::OP_C, C8(3), P));
  zconvert_or_copy<TC>(n, P, C8(3), SigL, s);
  // H00 = Hii(1) + sigma_r_ph(1) S ;  g_1 = (z S - H00 - Sigma_L)^-1
  BatchRef H00 = T(0);
  qt::zaxpby<TC>(n, P, HII(0), 1, 0, SIGR(0), 1, 0, nullref(), H00, nullptr, s);
  qt::zaxpby<TC>(n, P, H00, -1, 0, SigL, -1, 0, Zi, T(3), nullptr, s);
  QT_TRY(op.inv(T(3), GL(0), P, status));
  // Sigma^< = -(Sigma_L - Sigma_L^+) f_L + sigma_lesser_ph S ;  g^<_1 = g Sigma^< g^+
  qt::zantiherm<TC>(n, P, SigL, -1, 0, nullref(), T(4), s);
  qt::zscale_add<TC>(n, P, T(4), fl, SIGL(0), T(4), s);
  QT_TRY(op.gemm(GL(0), qt::OP_N, T(4), qt::OP_N, T(5), P));
  QT_TRY(op.gemm(T(5), qt::OP_N, GL(0), qt::OP_C, GLN(0), P));
  if (caroli) qt::zcopy<TC>(n, P, GL(0), Pch, s);  // P_0 = g_0

  // ---------------- forward sweep (src/cuda_rgf_mod.f90:140-188)
  for (int l = 1; l <= nx - 2; ++l) {
    const BatchRef H10 = H1I(l);
    // A = z S - (Hii + sigma_r_ph) - H10 g_{l-1} H10^+   (sigma_r_ph without *S, :142)
    QT_TRY(op.gemm(H10, qt::OP_N, GL(l - 1), qt::OP_N, T(0), P));
    if (pb.sigr) {
      qt::zaxpby<TC>(n, P, HII(l), 1, 0, SIGR(l), 1, 0, nullref(), T(2), nullptr, s);
      QT_TRY(op.gemm(T(0), qt::OP_N, H10, qt::OP_C, T(1), P, mone, T(2), mone, Zi));
    } else {
      QT_TRY(op.gemm(T(0), qt::OP_N, H10, qt::OP_C, T(1), P, mone, HII(l), mone, Zi));
    }
    QT_TRY(op.inv(T(1), GL(l), P, status));
    if (!pb.sigl) {
      // ballistic: g^<_l = M g^<_{l-1} M^+ and P_l = M P_{l-1} with M = g_l H_{l,l-1}
      // (4 block products where the general form below takes 6)
      const BatchRef M = T(1);
      QT_TRY(op.gemm(GL(l), qt::OP_N, H10, qt::OP_N, M, P));
      QT_TRY(op.gemm(GLN(l - 1), qt::OP_N, M, qt::OP_C, T(0), P));
      QT_TRY(op.gemm(M, qt::OP_N, T(0), qt::OP_N, GLN(l), P));
      if (caroli) {
        QT_TRY(op.gemm(M, qt::OP_N, Pch, qt::OP_N, Pnext, P));
        std::swap(Pch, Pnext);
      }
    } else {
      // g^<_l = g (H10 g^<_{l-1} H10^+ + sigma_lesser_ph S) g^+
      QT_TRY(op.gemm(H10, qt::OP_N, GLN(l - 1), qt::OP_N, T(0), P));
      QT_TRY(op.gemm(T(0), qt::OP_N, H10, qt::OP_C, T(1), P, one_c, SIGL(l), one_c));
      QT_TRY(op.gemm(GL(l), qt::OP_N, T(1), qt::OP_N, T(0), P));
      QT_TRY(op.gemm(T(0), qt::OP_N, GL(l), qt::OP_C, GLN(l), P));
      if (caroli) {  // P_l = g_l H_{l,l-1} P_{l-1}
        QT_TRY(op.gemm(H10, qt::OP_N, Pch, qt::OP_N, T(0), P));
        QT_TRY(op.gemm(GL(l), qt::OP_N, T(0), qt::OP_N, Pnext, P));
        std::swap(Pch, Pnext);
      }
    }
  }

  // ---------------- right contact (src/cuda_rgf_mod.f90:192-277)
  const BatchRef H10 = H1I(N);  // the reference uses H1i(nx) (1-based) for the right lead
  // Sigma_R = H10^+ G00 H10 at FP64 grade (G00 of the right lead: C8(5))
  QT_TRY(cop.gemm(H1I8(N), qt::OP_C, C8(5), qt::OP_N, C8(2), P));
  QT_TRY(cop.gemm(C8(2), qt::OP_N, H1I8(N), qt::OP_N, C8(3), P));
  const BatchRef SigR = T(2);
  zconvert_or_copy<TC>(n, P, C8(3), SigR, s);
  // G_NN = (z S - H00 - Sigma_R - H10 g_{N-1} H10^+)^-1
  qt::zaxpby<TC>(n, P, HII(N), 1, 0, SIGR(N), 1, 0, nullref(), T(0), nullptr, s);  // H00
  QT_TRY(op.gemm(H10, qt::OP_N, GL(N - 1), qt::OP_N, T(3), P));
  qt::zaxpby<TC>(n, P, T(0), -1, 0, SigR, -1, 0, Zi, T(4), nullptr, s);
  QT_TRY(op.gemm(T(3), qt::OP_N, H10, qt::OP_C, T(5), P, mone, T(4), one_c));
  BatchRef Gcur = T(6), Gncur = T(7), Gpcur = T(8), Gnew = T(3), Gnnew = T(4), Gpnew = T(11);
  QT_TRY(op.inv(T(5), Gcur, P, status));
  // Sigma^< = Gamma'_R f_R + H10 g^<_{N-1} H10^+ + sigma_lesser_ph S,  Gamma' = -(Sigma - Sigma^+)
  const BatchRef GamR = T(9);
  qt::zantiherm<TC>(n, P, SigR, -1, 0, nullref(), GamR, s);
  QT_TRY(op.gemm(H10, qt::OP_N, GLN(N - 1), qt::OP_N, T(0), P));
  QT_TRY(op.gemm(T(0), qt::OP_N, H10, qt::OP_C, T(5), P, one_c, SIGL(N), one_c));
  qt::zscale_add<TC>(n, P, GamR, fr, T(5), T(5), s);
  QT_TRY(op.gemm(Gcur, qt::OP_N, T(5), qt::OP_N, T(0), P));
  QT_TRY(op.gemm(T(0), qt::OP_N, Gcur, qt::OP_C, Gncur, P));
  // G^>_NN = G^< + (G - G^+)   (src/cuda_rgf_mod.f90:254)
  qt::zantiherm<TC>(n, P, Gcur, 1, 0, Gncur, Gpcur, s);
  if (pb.tr) qt::ztrace_current<TC>(n, P, SigR, Gpcur, Gncur, tr_sign, fr, pb.tr + p0, s);
  if (caroli) {
    // G_N1 = G_NN H_{N,N-1} P_{N-1};  T = Re Tr[Gam_R G_N1 Gam_L G_N1^+] with Gam = i(S - S^+)
    //   = -Re Tr[Gam'_R G_N1 Gam'_L G_N1^+]
    QT_TRY(op.gemm(H10, qt::OP_N, Pch, qt::OP_N, T(0), P));
    QT_TRY(op.gemm(Gcur, qt::OP_N, T(0), qt::OP_N, T(10), P));  // G_N1
    qt::zantiherm<TC>(n, P, SigL, -1, 0, nullref(), T(5), s);     // Gam'_L
    QT_TRY(op.gemm(T(5), qt::OP_N, T(10), qt::OP_C, T(0), P));  // Gam'_L G_N1^+
    QT_TRY(op.gemm(T(10), qt::OP_N, T(0), qt::OP_N, T(5), P));  // G_N1 Gam'_L G_N1^+
    qt::ztrace_prod<TC>(n, P, GamR, T(5), -1.0, pb.T + p0, s);
  }
  const bool glp = (q & QT_QUIRK_GLP_ZERO) != 0;
  auto emit = [&](int l, BatchRef G, BatchRef Gn, BatchRef Gp) {
    const long long os = (long long)nx * n, oo = (long long)l * n;
    if (pb.dgr) qt::zdiag<TC>(n, P, G, pb.dgr + 2 * p0 * nx * n, os, oo, s);
    if (pb.dgl) qt::zdiag<TC>(n, P, Gn, pb.dgl + 2 * p0 * nx * n, os, oo, s);
    if (pb.dgg) {
      if (glp) qt::zdiag<TC>(n, P, Gp, pb.dgg + 2 * p0 * nx * n, os, oo, s);
      else qt::zdiag_greater<TC>(n, P, G, Gn, pb.dgg + 2 * p0 * nx * n, os, oo, s);
    }
    if (pb.Gr) to_c128<TC>(n, P, G, OUTB(pb.Gr, l), s);
    if (pb.Gl) to_c128<TC>(n, P, Gn, OUTB(pb.Gl, l), s);
    if (pb.Gg) {
      if (glp) {
        to_c128<TC>(n, P, Gp, OUTB(pb.Gg, l), s);
      } else {
        qt::zantiherm<TC>(n, P, G, 1, 0, Gn, T(9), s);  // T(9) is free once emitting
        to_c128<TC>(n, P, T(9), OUTB(pb.Gg, l), s);
      }
    }
  };
  emit(N, Gcur, Gncur, Gpcur);
  if (pb.Jd)  // Jdens(nx) keeps its zero initialisation (src/cuda_rgf_mod.f90:84,283)
    cudaMemset2DAsync(pb.Jd + (p0 * nx + N) * nm2, (size_t)nx * nm2 * sizeof(cd), 0,
                      (size_t)nm2 * sizeof(cd), P, s);

  // ---------------- backward sweep (src/cuda_rgf_mod.f90:283-381)
  //   X = g H^+ ; GN0 = X G_{l+1} ; Y = GN0 H ; G_l = g + Y g
  //   G^<_l = g^< + X G^<_{l+1} X^+ + W - W^+ ,  W = Y g^<
  // The reference's fourth term g^< H^+ GN0^+ (:346-348) equals -W^+ because
  // g^< is anti-Hermitian, and GN0 (H g) = (GN0 H) g shares Y with W: 7 block
  // products per slab where the reference forms 30.
  for (int l = N - 1; l >= 0; --l) {
    const BatchRef Hc = (q & QT_QUIRK_BACK_H1I_NEXT) ? H1I(l + 1) : H1I(l);
    const BatchRef X = T(0), GN0 = T(1), Y = T(2), T1 = T(5), W = T(10);
    QT_TRY(op.gemm(GL(l), qt::OP_N, Hc, qt::OP_C, X, P));
    QT_TRY(op.gemm(X, qt::OP_N, Gcur, qt::OP_N, GN0, P));
    QT_TRY(op.gemm(GN0, qt::OP_N, Hc, qt::OP_N, Y, P));
    QT_TRY(op.gemm(Y, qt::OP_N, GL(l), qt::OP_N, Gnew, P, one_c, GL(l), one_c));
    QT_TRY(op.gemm(X, qt::OP_N, Gncur, qt::OP_N, T1, P));
    QT_TRY(op.gemm(T1, qt::OP_N, X, qt::OP_C, Gnnew, P, one_c, GLN(l), one_c));
    QT_TRY(op.gemm(Y, qt::OP_N, GLN(l), qt::OP_N, W, P));
    qt::zantiherm<TC>(n, P, W, 1, 0, Gnnew, Gnnew, s);
    if (pb.bond || pb.Jd) {
      // Bond current l -> l+1 (src/cuda_rgf_mod.f90:293-318):
      //   cur = H^+ B - H G^<_{l,l+1} = H^+ B + H B^+,  B = G^<_{l+1,l} = G^<_{l+1} X^+ + G_{l+1} U,
      //   U = H g^<_l, with G^<_{l,l+1} = -B^+ by anti-Hermiticity of G^<.
      // The CPU routine's form (src/rgf_mod.f90:215-221) is cur = -2 H^+ B.
      // Its trace only needs A = G_{l+1} U: Re Tr[H^+ G^<_{l+1} H g^+] = -Re Tr[T1 H]
      // with T1 = X G^<_{l+1} from the G^< update, so Re Tr cur = 2 (-Re Tr[T1 H] + Re Tr[H^+ A]).
      const double jsign = (q & QT_QUIRK_CPU_FERMI) ? -1.0 : 1.0;
      const long long bo = (long long)(nx - 1);
      QT_TRY(op.gemm(Hc, qt::OP_N, GLN(l), qt::OP_N, T(2), P));  // U
      QT_TRY(op.gemm(Gcur, qt::OP_N, T(2), qt::OP_N, T(1), P));  // A = G_{l+1} U
      if (pb.Jd) {
        QT_TRY(op.gemm(Gncur, qt::OP_N, X, qt::OP_C, T(2), P, one_c, T(1), one_c));  // B
        QT_TRY(op.gemm(Hc, qt::OP_C, T(2), qt::OP_N, W, P));                          // H^+ B
        QT_TRY(op.gemm(Hc, qt::OP_N, T(2), qt::OP_C, T(1), P, one_c, W, one_c));      // + H B^+
        to_c128<TC>(n, P, T(1), OUTB(pb.Jd, l), s);
        if (pb.bond)
          qt::zbond_trace<TC>(n, n, P, nullref(), Hc, T(2), jsign, pb.bond + p0 * bo, bo, l, s);
      } else {
        qt::zbond_trace<TC>(n, n, P, T1, Hc, T(1), jsign, pb.bond + p0 * bo, bo, l, s);
      }
    }
    if (glp) {  // G^>_l = X G^>_{l+1} X^+ (Glp never filled, src/cuda_rgf_mod.f90:78,351-372)
      QT_TRY(op.gemm(X, qt::OP_N, Gpcur, qt::OP_N, T1, P));
      QT_TRY(op.gemm(T1, qt::OP_N, X, qt::OP_C, Gpnew, P));
      std::swap(Gpcur, Gpnew);
    }
    std::swap(Gcur, Gnew);
    std::swap(Gncur, Gnnew);
    emit(l, Gcur, Gncur, Gpcur);
  }
  // ---------------- left-contact current tre (src/cuda_rgf_mod.f90:387-407)
  if (pb.tre) {
    qt::zantiherm<TC>(n, P, Gcur, 1, 0, Gncur, T(0), s);  // G^>_1 = G^< + (G - G^+)
    qt::ztrace_current<TC>(n, P, SigL, T(0), Gncur, 1.0, fe, pb.tre + p0, s);
  }
  qt::zcheck_finite<TC>(n, P, Gcur, status, s);  // canary on the last block touched
  check_wave_outputs(P, (long long)nx * n, p0, pb.dgr, pb.dgl, pb.dgg, pb.T, pb.tr, pb.tre,
                     status, s);
  if (pb.status)
    cudaMemcpyAsync(pb.status + p0, status, P * sizeof(int), cudaMemcpyDeviceToDevice, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

// ------------------------------------------------- variable block sizes
// Slabs of different orbital counts n_l (rgf_variableblock_forward,
// src/rgf_mod.f90:46-269).  H1i[l] = H_{l,l-1} is n_l x n_{l-1}; H1i[0] and
// H1i[nx] are the leads' own couplings (n_0 x n_0, n_{nx-1} x n_{nx-1}).  The
// backward step couples slab l to l+1 through H_{l+1,l} = H1i[l+1] (the
// reference's H1i(l) only fits equal neighbouring blocks), and the right lead is
// decimated with H1i[nx] as in the CPU routine (src/rgf_mod.f90:153).
struct ProblemVB {
  int nx, nk, nmax;
  long long npts, dsum;             // points; sum of n_l (diagonal output stride)
  std::vector<int> n;               // [nx]
  std::vector<long long> hoff, h1off, doff, goff;  // H / H1i offsets, diagonal and g offsets
  long long gsum;                   // sum of n_l^2
  const cd* Hii; long long hk;
  const cd* H1i; long long h1k;
  const float2* Hii32;
  const float2* H1i32;
  const double* E;
  qt_contacts c;
  qt_precision prec;
  unsigned flags;
  int sweep_slices, lead_slices, sweep_refine;
  double *tr, *tre, *T, *dgr, *dgl, *dgg;
  double* bond;  // [npts][nx-1] bond currents
  int *status, *iters;
};

size_t wave_bytes_vb(const ProblemVB& pb, long long P) {
  const size_t m2 = (size_t)pb.nmax * pb.nmax;
  const size_t tc = pb.prec == QT_PREC_MIXED ? 8 : 16;
  const size_t sweep = (2 * (size_t)pb.gsum + 16 * m2) * tc;
  const size_t lead = (7 + 2 + 6) * 16 * m2;
  const size_t guard = tc == 8 ? 16 * m2 : 0;  // complex128 workspace of the inverse guard
  return (sweep + lead + guard) * P + (size_t)P * (512 + 2048 + 8) + (512 << 10);
}

template <typename TC>
qt_status solve_wave_vb(qt_ctx* ctx, const ProblemVB& pb, long long p0, long long P, Arena& ar) {
  const int nx = pb.nx, nk = pb.nk, nm = pb.nmax;
  const long long m2 = (long long)nm * nm;
  cudaStream_t s = ctx->stream;
  const unsigned q = pb.c.quirks;
  const bool split = pb.prec != QT_PREC_FP64;
  const bool c64 = sizeof(TC) == 8;
  const std::vector<int>& n = pb.n;

  cd* zint = ar.take<cd>(P);
  cd* zlead = ar.take<cd>(P);
  double* fl = ar.take<double>(P);
  double* fr = ar.take<double>(P);
  double* fe = ar.take<double>(P);
  cd* one = ar.take<cd>(1);
  int* status = ar.take<int>(P);
  TC* gl_all = ar.take<TC>((size_t)pb.gsum * P);   // g_l   [l][b][n_l^2]
  TC* gln_all = ar.take<TC>((size_t)pb.gsum * P);  // g^<_l
  TC* tmp = ar.take<TC>((size_t)14 * P * m2);
  TC* rt1 = ar.take<TC>((size_t)P * m2);
  TC* rt2 = ar.take<TC>((size_t)P * m2);
  cd* cbuf = ar.take<cd>((size_t)6 * P * m2);
  int* scales = ar.take<int>((size_t)P * 256);
  unsigned char* guard = ar.take<unsigned char>((size_t)P);
  cd* fbw = c64 ? ar.take<cd>((size_t)P * m2) : nullptr;
  if (!zint || !zlead || !fl || !fr || !fe || !one || !status || !gl_all || !gln_all || !tmp ||
      !rt1 || !rt2 || !cbuf || !scales || !guard || (c64 && !fbw))
    QT_FAIL(QT_ERR_NOMEM, "wave arena exhausted");
  Ops<TC> op{s, nm, pb.prec};
  op.slices = pb.sweep_slices;
  op.refine = split ? pb.sweep_refine : 0;
  op.one = one; op.rt1 = rt1; op.rt2 = rt2; op.P = P; op.scales = scales;
  op.prof = &ctx->prof;
  op.guard = guard; op.fbw = fbw; op.fallbacks = ctx->fallbacks;
  Ops<double2> cop{s, nm, pb.prec};
  cop.prof = &ctx->prof;
  cop.slices = pb.lead_slices;
  cop.refine = split ? 3 : 0;
  cop.one = one; cop.scales = scales; cop.P = P;
  cop.guard = guard; cop.fallbacks = ctx->fallbacks;

  const cd h1{1.0, 0.0};
  cudaMemcpyAsync(one, &h1, sizeof(cd), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(status, 0, P * sizeof(int), s);
  make_z_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, pb.c.eta_interior, zint);
  qt::count_launch();
  make_z_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, pb.c.eta_lead, zlead);
  qt::count_launch();
  const bool cpu = (q & QT_QUIRK_CPU_FERMI) != 0;
  make_fermi_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, cpu ? pb.c.mur : pb.c.mul,
                                           cpu ? pb.c.tempr : pb.c.templ, fl);
  qt::count_launch();
  make_fermi_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, cpu ? pb.c.mul : pb.c.mur, pb.c.templ,
                                           fr);
  qt::count_launch();
  make_fermi_kernel<<<g1d(P), 256, 0, s>>>(pb.E, p0, P, nk, cpu ? pb.c.mur : pb.c.mul, pb.c.tempr,
                                           fe);
  qt::count_launch();
  const double tr_sign = cpu ? 1.0 : -1.0;

  // temporaries hold up to nmax x nmax per point; ld = rows of what they hold
  auto T = [&](int i, int ld) { return ref(tmp + (size_t)i * P * m2, m2, ld); };
  auto C8 = [&](int i, int ld) { return ref(cbuf + (size_t)i * P * m2, m2, ld); };
  auto GL = [&](int l) {
    return ref(gl_all + (size_t)pb.goff[l] * P, (long long)n[l] * n[l], n[l]);
  };
  auto GLN = [&](int l) {
    return ref(gln_all + (size_t)pb.goff[l] * P, (long long)n[l] * n[l], n[l]);
  };
  auto HII8 = [&](int l) { return ref(pb.Hii + pb.hoff[l], pb.hk, n[l], pb.hk ? nk : 0); };
  auto HII = [&](int l) {
    return c64 ? ref(pb.Hii32 + pb.hoff[l], pb.hk, n[l], pb.hk ? nk : 0) : HII8(l);
  };
  // coupling l: rows n_l (n_0 / n_{nx-1} for the leads' own couplings)
  auto rows1 = [&](int l) { return l == 0 ? n[0] : (l == nx ? n[nx - 1] : n[l]); };
  auto H1I8 = [&](int l) { return ref(pb.H1i + pb.h1off[l], pb.h1k, rows1(l), pb.h1k ? nk : 0); };
  auto H1I = [&](int l) {
    return c64 ? ref(pb.H1i32 + pb.h1off[l], pb.h1k, rows1(l), pb.h1k ? nk : 0) : H1I8(l);
  };
  const BatchRef Zi = ref(zint, 1, 1);
  const cd one_c{1, 0}, mone{-1, 0};
  const bool caroli = (pb.flags & QT_FLAG_CAROLI) && pb.T;
  const int n0 = n[0], N = nx - 1, nN = n[N];
  auto emit = [&](int l, BatchRef G, BatchRef Gn) {
    const long long os = pb.dsum, oo = pb.doff[l];
    if (pb.dgr) qt::zdiag<TC>(n[l], P, G, pb.dgr + 2 * p0 * pb.dsum, os, oo, s);
    if (pb.dgl) qt::zdiag<TC>(n[l], P, Gn, pb.dgl + 2 * p0 * pb.dsum, os, oo, s);
    if (pb.dgg) qt::zdiag_greater<TC>(n[l], P, G, Gn, pb.dgg + 2 * p0 * pb.dsum, os, oo, s);
  };

  // ---------------- left contact: lead block n_0 with its own coupling H1i[0]
  {
    Ops<double2> lop = cop;
    lop.n = n0;
    QT_TRY(sancho_wave(lop, ar, P, HII8(0), H1I8(0), true, zlead, pb.c.sancho_tol,
                       pb.c.sancho_max_iter, C8(1, n0), nullref(), status,
                       pb.iters ? pb.iters + p0 * 2 : nullptr, 2, nullref(),
                       (pb.c.quirks & QT_QUIRK_GW_SANCHO_RESET) != 0));
    QT_TRY(cop.gemm3(n0, n0, n0, H1I8(0), qt::OP_N, C8(1, n0), qt::OP_N, C8(2, n0), P));
    QT_TRY(cop.gemm3(n0, n0, n0, C8(2, n0), qt::OP_N, H1I8(0), qt::OP_C, C8(3, n0), P));
  }
  const BatchRef SigL = T(13, n0);
  int pc = 12;  // temporary holding the Caroli chain P_l (ping-pongs with 11)
  zconvert_or_copy<TC>(n0, P, C8(3, n0), SigL, s);
  qt::zaxpby<TC>(n0, P, HII(0), -1, 0, SigL, -1, 0, Zi, T(3, n0), nullptr, s);
  QT_TRY(op.inv(T(3, n0), GL(0), P, status, nullptr, n0));
  qt::zantiherm<TC>(n0, P, SigL, -1, 0, nullref(), T(4, n0), s);
  qt::zscale_add<TC>(n0, P, T(4, n0), fl, nullref(), T(4, n0), s);
  QT_TRY(op.gemm3(n0, n0, n0, GL(0), qt::OP_N, T(4, n0), qt::OP_N, T(5, n0), P));
  QT_TRY(op.gemm3(n0, n0, n0, T(5, n0), qt::OP_N, GL(0), qt::OP_C, GLN(0), P));
  // Caroli chain P_l (n_l x n_0), ld n_l
  if (caroli) qt::zcopy<TC>(n0, P, GL(0), ref(tmp + (size_t)12 * P * m2, m2, n0), s);

  // ---------------- forward sweep
  for (int l = 1; l <= N - 1; ++l) {
    const int nl = n[l], np = n[l - 1];
    const BatchRef H10 = H1I(l);  // n_l x n_{l-1}
    QT_TRY(op.gemm3(nl, np, np, H10, qt::OP_N, GL(l - 1), qt::OP_N, T(0, nl), P));
    QT_TRY(op.gemm3(nl, nl, np, T(0, nl), qt::OP_N, H10, qt::OP_C, T(1, nl), P, mone, HII(l),
                    mone, Zi));
    QT_TRY(op.inv(T(1, nl), GL(l), P, status, nullptr, nl));
    // g^<_l = M g^<_{l-1} M^+ and P_l = M P_{l-1} with M = g_l H_{l,l-1} (n_l x n_{l-1})
    QT_TRY(op.gemm3(nl, np, nl, GL(l), qt::OP_N, H10, qt::OP_N, T(1, nl), P));
    QT_TRY(op.gemm3(np, nl, np, GLN(l - 1), qt::OP_N, T(1, nl), qt::OP_C, T(0, np), P));
    QT_TRY(op.gemm3(nl, nl, np, T(1, nl), qt::OP_N, T(0, np), qt::OP_N, GLN(l), P));
    if (caroli) {  // the chain ping-pongs between temporaries 12 and 11
      QT_TRY(op.gemm3(nl, n0, np, T(1, nl), qt::OP_N, ref(tmp + (size_t)pc * P * m2, m2, np),
                      qt::OP_N, ref(tmp + (size_t)(23 - pc) * P * m2, m2, nl), P));
      pc = 23 - pc;
    }
  }

  // ---------------- right contact: lead block n_N, decimated with its own H1i[nx]
  {
    Ops<double2> lop = cop;
    lop.n = nN;
    QT_TRY(sancho_wave(lop, ar, P, HII8(N), H1I8(nx), false, zlead, pb.c.sancho_tol,
                       pb.c.sancho_max_iter, C8(1, nN), nullref(), status,
                       pb.iters ? pb.iters + p0 * 2 + 1 : nullptr, 2, nullref(),
                       (pb.c.quirks & QT_QUIRK_GW_SANCHO_RESET) != 0));
    QT_TRY(cop.gemm3(nN, nN, nN, H1I8(nx), qt::OP_C, C8(1, nN), qt::OP_N, C8(2, nN), P));
    QT_TRY(cop.gemm3(nN, nN, nN, C8(2, nN), qt::OP_N, H1I8(nx), qt::OP_N, C8(3, nN), P));
  }
  const BatchRef SigR = T(2, nN);
  zconvert_or_copy<TC>(nN, P, C8(3, nN), SigR, s);
  const int np = n[N - 1];
  const BatchRef Hd = H1I(N);  // device coupling n_N x n_{N-1}
  QT_TRY(op.gemm3(nN, np, np, Hd, qt::OP_N, GL(N - 1), qt::OP_N, T(3, nN), P));
  qt::zaxpby<TC>(nN, P, HII(N), -1, 0, SigR, -1, 0, Zi, T(4, nN), nullptr, s);
  QT_TRY(op.gemm3(nN, nN, np, T(3, nN), qt::OP_N, Hd, qt::OP_C, T(5, nN), P, mone, T(4, nN),
                  one_c));
  int ig = 6, ign = 7, inew = 3, innew = 4;  // rotating temporaries for G, G^<
  QT_TRY(op.inv(T(5, nN), T(ig, nN), P, status, nullptr, nN));
  const BatchRef GamR = T(9, nN);
  qt::zantiherm<TC>(nN, P, SigR, -1, 0, nullref(), GamR, s);
  QT_TRY(op.gemm3(nN, np, np, Hd, qt::OP_N, GLN(N - 1), qt::OP_N, T(0, nN), P));
  QT_TRY(op.gemm3(nN, nN, np, T(0, nN), qt::OP_N, Hd, qt::OP_C, T(5, nN), P));
  qt::zscale_add<TC>(nN, P, GamR, fr, T(5, nN), T(5, nN), s);
  QT_TRY(op.gemm3(nN, nN, nN, T(ig, nN), qt::OP_N, T(5, nN), qt::OP_N, T(0, nN), P));
  QT_TRY(op.gemm3(nN, nN, nN, T(0, nN), qt::OP_N, T(ig, nN), qt::OP_C, T(ign, nN), P));
  qt::zantiherm<TC>(nN, P, T(ig, nN), 1, 0, T(ign, nN), T(8, nN), s);  // G^>_NN
  if (pb.tr) qt::ztrace_current<TC>(nN, P, SigR, T(8, nN), T(ign, nN), tr_sign, fr, pb.tr + p0, s);
  if (caroli) {
    // G_N1 = G_NN H_{N,N-1} P_{N-1} (n_N x n_0); T = -Re Tr[Gam'_R G_N1 Gam'_L G_N1^+]
    QT_TRY(op.gemm3(nN, n0, np, Hd, qt::OP_N, ref(tmp + (size_t)pc * P * m2, m2, np), qt::OP_N,
                    T(0, nN), P));
    QT_TRY(op.gemm3(nN, n0, nN, T(ig, nN), qt::OP_N, T(0, nN), qt::OP_N, T(10, nN), P));
    qt::zantiherm<TC>(n0, P, SigL, -1, 0, nullref(), T(5, n0), s);
    QT_TRY(op.gemm3(n0, nN, n0, T(5, n0), qt::OP_N, T(10, nN), qt::OP_C, T(0, n0), P));
    QT_TRY(op.gemm3(nN, nN, n0, T(10, nN), qt::OP_N, T(0, n0), qt::OP_N, T(5, nN), P));
    qt::ztrace_prod<TC>(nN, P, GamR, T(5, nN), -1.0, pb.T + p0, s);
  }
  emit(N, T(ig, nN), T(ign, nN));

  // ---------------- backward sweep, coupling H_{l+1,l} = H1i[l+1] (n_{l+1} x n_l)
  for (int l = N - 1; l >= 0; --l) {
    const int nl = n[l], nq = n[l + 1];
    const BatchRef Hc = H1I(l + 1);
    // X = g H^+ (nl x nq); GN0 = X G_{l+1}; Y = GN0 H (nl x nl); G_l = g + Y g
    QT_TRY(op.gemm3(nl, nq, nl, GL(l), qt::OP_N, Hc, qt::OP_C, T(0, nl), P));
    QT_TRY(op.gemm3(nl, nq, nq, T(0, nl), qt::OP_N, T(ig, nq), qt::OP_N, T(1, nl), P));
    QT_TRY(op.gemm3(nl, nl, nq, T(1, nl), qt::OP_N, Hc, qt::OP_N, T(2, nl), P));
    QT_TRY(op.gemm3(nl, nl, nl, T(2, nl), qt::OP_N, GL(l), qt::OP_N, T(inew, nl), P, one_c,
                    GL(l), one_c));
    // G^<_l = g^< + X G^<_{l+1} X^+ + W - W^+,  W = Y g^<
    QT_TRY(op.gemm3(nl, nq, nq, T(0, nl), qt::OP_N, T(ign, nq), qt::OP_N, T(5, nl), P));
    QT_TRY(op.gemm3(nl, nl, nq, T(5, nl), qt::OP_N, T(0, nl), qt::OP_C, T(innew, nl), P, one_c,
                    GLN(l), one_c));
    QT_TRY(op.gemm3(nl, nl, nl, T(2, nl), qt::OP_N, GLN(l), qt::OP_N, T(10, nl), P));
    qt::zantiherm<TC>(nl, P, T(10, nl), 1, 0, T(innew, nl), T(innew, nl), s);
    if (pb.bond) {
      // bond current l -> l+1, trace form of the solve path: U = H g^< (nq x nl),
      // A = G_{l+1} U, out = sign 2 (-Re Tr[T1 H] + Re Tr[H^+ A]), T1 = X G^<_{l+1} (nl x nq)
      const double jsign = (q & QT_QUIRK_CPU_FERMI) ? -1.0 : 1.0;
      QT_TRY(op.gemm3(nq, nl, nl, Hc, qt::OP_N, GLN(l), qt::OP_N, T(2, nq), P));
      QT_TRY(op.gemm3(nq, nl, nq, T(ig, nq), qt::OP_N, T(2, nq), qt::OP_N, T(1, nq), P));
      qt::zbond_trace<TC>(nl, nq, P, T(5, nl), Hc, T(1, nq), jsign, pb.bond + p0 * (nx - 1),
                          nx - 1, l, s);
    }
    std::swap(ig, inew);
    std::swap(ign, innew);
    emit(l, T(ig, nl), T(ign, nl));
  }
  if (pb.tre) {
    qt::zantiherm<TC>(n0, P, T(ig, n0), 1, 0, T(ign, n0), T(0, n0), s);
    qt::ztrace_current<TC>(n0, P, SigL, T(0, n0), T(ign, n0), 1.0, fe, pb.tre + p0, s);
  }
  qt::zcheck_finite<TC>(n0, P, T(ig, n0), status, s);
  check_wave_outputs(P, pb.dsum, p0, pb.dgr, pb.dgl, pb.dgg, pb.T, pb.tr, pb.tre, status, s);
  if (pb.status)
    cudaMemcpyAsync(pb.status + p0, status, P * sizeof(int), cudaMemcpyDeviceToDevice, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

// choose the wave size: a multiple of nk, bounded by the scratch limit
long long choose_wave(const qt_ctx* ctx, const Problem& pb) {
  const size_t per = wave_bytes(pb, 1);
  long long P = (long long)((size_t)ctx->scratch_limit / (per + 1));
  // several work items per SM in every batched launch unless the context sets the wave
  const long long target = ctx->wave_points > 0 ? ctx->wave_points : 152 * 4;
  P = std::min<long long>(P, std::max<long long>(target, pb.nk));
  P = std::min<long long>(P, pb.npts);
  P = std::max<long long>(P / pb.nk, 1) * pb.nk;
  return P;
}

struct HostStage {
  // copy helper for host-pointer calls
  qt_ctx* ctx;
  char* base = nullptr;
  size_t off = 0;
  template <typename T>
  T* put(const T* src, size_t count, bool copy) {
    if (!src && copy) return nullptr;
    T* d = reinterpret_cast<T*>(base + off);
    off += (count * sizeof(T) + 255) & ~size_t(255);
    if (copy) cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
    return d;
  }
};

}  // namespace

// ============================================================== C-ABI
extern "C" qt_status qt_ctx_create(qt_ctx** out, int device) {
  if (!out) QT_FAIL(QT_ERR_ARG, "null ctx pointer");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    QT_FAIL(QT_ERR_CUDA, "no CUDA device");
  }
  if (device < 0 || device >= count) QT_FAIL(QT_ERR_ARG, "bad device index");
  qt_ctx* c = new qt_ctx();
  c->device = device;
  cudaSetDevice(device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    QT_FAIL(QT_ERR_CUDA, "stream creation failed");
  }
  c->stream = c->own_stream;
  if (cudaMalloc(&c->fallbacks, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->fallbacks, 0, sizeof(int)) != cudaSuccess) {
    cudaStreamDestroy(c->own_stream);
    delete c;
    QT_FAIL(QT_ERR_CUDA, "context counter allocation failed");
  }
  *out = c;
  return QT_OK;
}

extern "C" qt_status qt_ctx_destroy(qt_ctx* c) {
  if (!c) return QT_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->arena) cudaFree(c->arena);
  if (c->io) cudaFree(c->io);
  if (c->conv) cudaFree(c->conv);
  if (c->fallbacks) cudaFree(c->fallbacks);
  for (auto& e : c->prof.v) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
  for (auto e : c->prof.pool) cudaEventDestroy(e);
  cudaStreamDestroy(c->own_stream);
  delete c;
  return QT_OK;
}

extern "C" qt_status qt_ctx_sync(qt_ctx* c) {
  if (!c) QT_FAIL(QT_ERR_ARG, "null ctx");
  QT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return QT_OK;
}

extern "C" qt_status qt_ctx_set_scratch_limit(qt_ctx* c, int64_t bytes) {
  if (!c || bytes <= 0) QT_FAIL(QT_ERR_ARG, "bad scratch limit");
  c->scratch_limit = bytes;
  return QT_OK;
}

extern "C" qt_status qt_ctx_set_wave_points(qt_ctx* c, int64_t points) {
  if (!c || points < 0) QT_FAIL(QT_ERR_ARG, "bad wave size");
  c->wave_points = points;
  return QT_OK;
}

extern "C" qt_status qt_ctx_set_gw_grid(qt_ctx* c, int nky, int nkz, int ndiag) {
  if (!c || nky < 1 || nkz < 1) QT_FAIL(QT_ERR_ARG, "need nky >= 1 and nkz >= 1");
  c->gw_nky = nky;
  c->gw_nkz = nkz;
  c->gw_ndiag = ndiag < 0 ? -1 : ndiag;
  return QT_OK;
}

extern "C" qt_status qt_ctx_profile(qt_ctx* c, int enable) {
  if (!c) QT_FAIL(QT_ERR_ARG, "null ctx");
  c->prof.on = enable != 0;
  return QT_OK;
}

extern "C" qt_status qt_ctx_profile_read(qt_ctx* c, int kind, int64_t* launches, double* ms,
                                         double* alg_flops, double* tensor_flops) {
  if (!c) QT_FAIL(QT_ERR_ARG, "null ctx");
  QT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  int64_t nl = 0;
  double t = 0.0, fa = 0.0, ft = 0.0;
  std::vector<Prof::Entry> keep;
  for (auto& e : c->prof.v) {
    if (e.kind != kind) { keep.push_back(e); continue; }
    float x = 0.f;
    cudaEventElapsedTime(&x, e.a, e.b);
    ++nl; t += x; fa += e.alg; ft += e.tensor;
    c->prof.pool.push_back(e.a);
    c->prof.pool.push_back(e.b);
  }
  c->prof.v.swap(keep);
  if (launches) *launches = nl;
  if (ms) *ms = t;
  if (alg_flops) *alg_flops = fa;
  if (tensor_flops) *tensor_flops = ft;
  return QT_OK;
}

extern "C" qt_status qt_ctx_set_stream(qt_ctx* c, void* stream, int use_own) {
  if (!c) QT_FAIL(QT_ERR_ARG, "null ctx");
  cudaSetDevice(c->device);
  QT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->stream = use_own ? c->own_stream : reinterpret_cast<cudaStream_t>(stream);
  return QT_OK;
}

extern "C" qt_status qt_ctx_inverse_fallbacks(qt_ctx* c, int64_t* count, int reset) {
  if (!c || !count) QT_FAIL(QT_ERR_ARG, "null argument");
  int h = 0;
  QT_CUDA_TRY(cudaMemcpyAsync(&h, c->fallbacks, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  QT_CUDA_TRY(cudaStreamSynchronize(c->stream));
  *count = h;
  if (reset) QT_CUDA_TRY(cudaMemsetAsync(c->fallbacks, 0, sizeof(int), c->stream));
  return QT_OK;
}

extern "C" qt_status qt_ctx_stream(qt_ctx* c, void** stream) {
  if (!c || !stream) QT_FAIL(QT_ERR_ARG, "null argument");
  *stream = (void*)c->stream;
  return QT_OK;
}

namespace {

bool valid_prec(qt_precision p) {
  return p == QT_PREC_FP64 || p == QT_PREC_MIXED || p == QT_PREC_MIXED_FP64;
}

int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return v && *v ? atoi(v) : dflt;
}

qt_status run_problem(qt_ctx* ctx, Problem& pb, long long hii_n, long long h1i_n) {
  // digits of the split-precision products: 4 for the complex64 sweep (MIXED), 6 for the
  // complex128 sweep (MIXED_FP64), 7 (FP64 grade) for the lead decimation;
  // QT_SWEEP_SLICES / QT_LEAD_SLICES override for accuracy studies
  const bool c64 = pb.prec == QT_PREC_MIXED;
  pb.sweep_slices = env_int("QT_SWEEP_SLICES", c64 ? 4 : 6);
  pb.lead_slices = env_int("QT_LEAD_SLICES", 7);
  // complex64 sweep: one refinement reaches its storage resolution; complex128 sweep
  // (MIXED_FP64): three, as for the leads.  QT_SWEEP_REFINE overrides.
  pb.sweep_refine = env_int("QT_SWEEP_REFINE", c64 ? 1 : 3);
  if (pb.sweep_refine < 0 || pb.sweep_refine > 8) QT_FAIL(QT_ERR_ARG, "QT_SWEEP_REFINE in 0..8");
  if (c64 && pb.sweep_slices != 3 && pb.sweep_slices != 4)
    QT_FAIL(QT_ERR_ARG, "QT_SWEEP_SLICES in {3,4} for the complex64 sweep");
  if (!c64 && pb.sweep_slices != 4 && pb.sweep_slices != 6 && pb.sweep_slices != 7)
    QT_FAIL(QT_ERR_ARG, "QT_SWEEP_SLICES in {4,6,7} for the complex128 sweep");
  if (pb.lead_slices != 4 && pb.lead_slices != 6 && pb.lead_slices != 7)
    QT_FAIL(QT_ERR_ARG, "QT_LEAD_SLICES in {4,6,7}");
  cudaStream_t s = ctx->stream;
  const bool split = pb.prec != QT_PREC_FP64;
  if (c64) {
    const long long blk = pb.npts * pb.nx * (long long)pb.nm * pb.nm;
    const long long cnt = hii_n + h1i_n + (pb.sigr ? blk : 0) + (pb.sigl ? blk : 0);
    QT_TRY(ensure(ctx->conv, ctx->conv_bytes, (size_t)cnt * sizeof(float2) + 4096));
    float2* c = reinterpret_cast<float2*>(ctx->conv);
    auto conv = [&](const cd* src, long long count) -> const float2* {
      if (!src) return nullptr;
      flat_d2f_kernel<<<g1d(count), 256, 0, s>>>(reinterpret_cast<const double2*>(src), c, count);
      qt::count_launch();
      const float2* r = c;
      c += count;
      return r;
    };
    pb.Hii32 = conv(pb.Hii, hii_n);
    pb.H1i32 = conv(pb.H1i, h1i_n);
    pb.sigr32 = conv(pb.sigr, blk);
    pb.sigl32 = conv(pb.sigl, blk);
  }
  const long long P = choose_wave(ctx, pb);
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, wave_bytes(pb, P)));
  for (long long p0 = 0; p0 < pb.npts; p0 += P) {
    const long long Pw = std::min(P, pb.npts - p0);
    Arena ar{reinterpret_cast<char*>(ctx->arena), ctx->arena_bytes, 0};
    if (c64) QT_TRY(solve_wave<float2>(ctx, pb, p0, Pw, ar));
    else QT_TRY(solve_wave<double2>(ctx, pb, p0, Pw, ar));
  }
  if (split) {
    QT_CUDA_TRY(cudaStreamSynchronize(s));
    if (qt::oz_timeouts_and_reset()) QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  }
  return QT_OK;
}

qt_status run_problem_vb(qt_ctx* ctx, ProblemVB& pb, long long hii_n, long long h1i_n) {
  const bool c64 = pb.prec == QT_PREC_MIXED;
  pb.sweep_slices = env_int("QT_SWEEP_SLICES", c64 ? 4 : 6);
  pb.lead_slices = env_int("QT_LEAD_SLICES", 7);
  pb.sweep_refine = env_int("QT_SWEEP_REFINE", c64 ? 1 : 3);
  if (pb.sweep_refine < 0 || pb.sweep_refine > 8) QT_FAIL(QT_ERR_ARG, "QT_SWEEP_REFINE in 0..8");
  if (c64 && pb.sweep_slices != 3 && pb.sweep_slices != 4)
    QT_FAIL(QT_ERR_ARG, "QT_SWEEP_SLICES in {3,4} for the complex64 sweep");
  if (!c64 && pb.sweep_slices != 4 && pb.sweep_slices != 6 && pb.sweep_slices != 7)
    QT_FAIL(QT_ERR_ARG, "QT_SWEEP_SLICES in {4,6,7} for the complex128 sweep");
  if (pb.lead_slices != 4 && pb.lead_slices != 6 && pb.lead_slices != 7)
    QT_FAIL(QT_ERR_ARG, "QT_LEAD_SLICES in {4,6,7}");
  cudaStream_t s = ctx->stream;
  if (c64) {
    QT_TRY(ensure(ctx->conv, ctx->conv_bytes, (size_t)(hii_n + h1i_n) * sizeof(float2) + 4096));
    float2* c = reinterpret_cast<float2*>(ctx->conv);
    flat_d2f_kernel<<<g1d(hii_n), 256, 0, s>>>(reinterpret_cast<const double2*>(pb.Hii), c, hii_n);
    qt::count_launch();
    flat_d2f_kernel<<<g1d(h1i_n), 256, 0, s>>>(reinterpret_cast<const double2*>(pb.H1i),
                                                c + hii_n, h1i_n);
    qt::count_launch();
    pb.Hii32 = c;
    pb.H1i32 = c + hii_n;
  }
  const size_t per = wave_bytes_vb(pb, 1);
  long long P = (long long)((size_t)ctx->scratch_limit / (per + 1));
  P = std::min<long long>(P, std::max<long long>(
                                 ctx->wave_points > 0 ? ctx->wave_points : 152 * 4, pb.nk));
  P = std::min<long long>(P, pb.npts);
  P = std::max<long long>(P / pb.nk, 1) * pb.nk;
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, wave_bytes_vb(pb, P)));
  for (long long p0 = 0; p0 < pb.npts; p0 += P) {
    const long long Pw = std::min(P, pb.npts - p0);
    Arena ar{reinterpret_cast<char*>(ctx->arena), ctx->arena_bytes, 0};
    if (c64) QT_TRY(solve_wave_vb<float2>(ctx, pb, p0, Pw, ar));
    else QT_TRY(solve_wave_vb<double2>(ctx, pb, p0, Pw, ar));
  }
  if (pb.prec != QT_PREC_FP64) {
    QT_CUDA_TRY(cudaStreamSynchronize(s));
    if (qt::oz_timeouts_and_reset()) QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  }
  return QT_OK;
}

}  // namespace

extern "C" qt_status qt_rgf_solve(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                                  const qt_contacts* c, const double* sigma_r_ph,
                                  const double* sigma_lesser_ph, qt_precision prec, unsigned flags,
                                  qt_outputs* out) {
  if (!ctx || !dev || !E || !c || !out) QT_FAIL(QT_ERR_ARG, "null argument");
  if (dev->nm <= 0 || dev->nx < 2 || dev->nk <= 0 || nE <= 0)
    QT_FAIL(QT_ERR_ARG, "need nm > 0, nx >= 2, nk > 0, nE > 0");
  if (!dev->Hii || !dev->H1i) QT_FAIL(QT_ERR_ARG, "Hii/H1i required");
  if (dev->Sii) QT_FAIL(QT_ERR_UNSUPPORTED, "Sii must be NULL (identity overlap)");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec != QT_PREC_FP64 && dev->nm > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "split-precision path needs nm <= 384");
  if (c->sancho_max_iter <= 0) QT_FAIL(QT_ERR_ARG, "sancho_max_iter must be > 0");
  if (out->Jdens && (c->quirks & QT_QUIRK_CPU_FERMI))
    QT_FAIL(QT_ERR_UNSUPPORTED, "Jdens blocks follow cuda_rgf_constblocksize (no QT_QUIRK_CPU_FERMI)");
  cudaSetDevice(ctx->device);
  const int nm = dev->nm, nx = dev->nx, nk = dev->nk;
  const long long npts = (long long)nE * nk;
  const long long nm2 = (long long)nm * nm;
  Problem pb{};
  pb.nm = nm; pb.nx = nx; pb.nk = nk; pb.npts = npts;
  pb.c = *c; pb.prec = prec; pb.flags = flags;
  pb.hk = dev->hii_kstride; pb.hl = dev->hii_lstride;
  pb.h1k = dev->h1i_kstride; pb.h1l = dev->h1i_lstride;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  // extents of the H arrays (elements) for host staging
  const long long hii_n = (pb.hk ? (nk - 1) * pb.hk : 0) + (pb.hl ? (nx - 1) * pb.hl : 0) + nm2;
  const long long h1i_n = (pb.h1k ? (nk - 1) * pb.h1k : 0) + (pb.h1l ? nx * pb.h1l : 0) + nm2;
  const long long blk_n = npts * nx * nm2;
  const long long diag_n = npts * nx * nm;
  HostStage st{ctx};
  if (devp) {
    pb.Hii = reinterpret_cast<const cd*>(dev->Hii);
    pb.H1i = reinterpret_cast<const cd*>(dev->H1i);
    pb.sigr = reinterpret_cast<const cd*>(sigma_r_ph);
    pb.sigl = reinterpret_cast<const cd*>(sigma_lesser_ph);
    pb.E = E;
    pb.tr = out->tr; pb.tre = out->tre; pb.T = out->T;
    pb.dgr = out->diag_gr; pb.dgl = out->diag_gl; pb.dgg = out->diag_gg;
    pb.Gr = reinterpret_cast<cd*>(out->G_r); pb.Gl = reinterpret_cast<cd*>(out->G_lesser);
    pb.Gg = reinterpret_cast<cd*>(out->G_greater);
    pb.bond = out->bond_cur; pb.Jd = reinterpret_cast<cd*>(out->Jdens);
    pb.status = out->status; pb.iters = out->sancho_iters;
    QT_TRY(run_problem(ctx, pb, hii_n, h1i_n));
  } else {
    size_t need = 0;
    auto add = [&](size_t bytes) { need += (bytes + 255) & ~size_t(255); };
    add(hii_n * 16); add(h1i_n * 16); add(nE * 8);
    if (sigma_r_ph) add(blk_n * 16);
    if (sigma_lesser_ph) add(blk_n * 16);
    add(npts * 8 * 3); add(diag_n * 16 * 3); add(npts * 4 * 3);
    if (out->G_r) add(blk_n * 16);
    if (out->G_lesser) add(blk_n * 16);
    if (out->G_greater) add(blk_n * 16);
    if (out->Jdens) add(blk_n * 16);
    if (out->bond_cur) add(npts * (nx - 1) * 8);
    QT_TRY(ensure(ctx->io, ctx->io_bytes, need + 4096));
    st.base = reinterpret_cast<char*>(ctx->io);
    pb.Hii = st.put(reinterpret_cast<const cd*>(dev->Hii), hii_n, true);
    pb.H1i = st.put(reinterpret_cast<const cd*>(dev->H1i), h1i_n, true);
    pb.E = st.put(E, nE, true);
    pb.sigr = sigma_r_ph ? st.put(reinterpret_cast<const cd*>(sigma_r_ph), blk_n, true) : nullptr;
    pb.sigl = sigma_lesser_ph ? st.put(reinterpret_cast<const cd*>(sigma_lesser_ph), blk_n, true) : nullptr;
    pb.tr = out->tr ? st.put<double>(nullptr, npts, false) : nullptr;
    pb.tre = out->tre ? st.put<double>(nullptr, npts, false) : nullptr;
    pb.T = out->T ? st.put<double>(nullptr, npts, false) : nullptr;
    pb.dgr = out->diag_gr || out->diag_gg ? st.put<double>(nullptr, 2 * diag_n, false) : nullptr;
    pb.dgl = out->diag_gl || out->diag_gg ? st.put<double>(nullptr, 2 * diag_n, false) : nullptr;
    pb.dgg = out->diag_gg ? st.put<double>(nullptr, 2 * diag_n, false) : nullptr;
    pb.Gr = out->G_r ? st.put<cd>(nullptr, blk_n, false) : nullptr;
    pb.Gl = out->G_lesser ? st.put<cd>(nullptr, blk_n, false) : nullptr;
    pb.Gg = out->G_greater ? st.put<cd>(nullptr, blk_n, false) : nullptr;
    pb.Jd = out->Jdens ? st.put<cd>(nullptr, blk_n, false) : nullptr;
    pb.bond = out->bond_cur ? st.put<double>(nullptr, npts * (nx - 1), false) : nullptr;
    pb.status = st.put<int>(nullptr, npts, false);
    pb.iters = st.put<int>(nullptr, 2 * npts, false);
    QT_TRY(run_problem(ctx, pb, hii_n, h1i_n));
    auto back = [&](void* dst, const void* src, size_t bytes) {
      if (dst && src) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    };
    back(out->tr, pb.tr, npts * 8);
    back(out->tre, pb.tre, npts * 8);
    back(out->T, pb.T, npts * 8);
    back(out->diag_gr, pb.dgr, diag_n * 16);
    back(out->diag_gl, pb.dgl, diag_n * 16);
    back(out->diag_gg, pb.dgg, diag_n * 16);
    back(out->G_r, pb.Gr, blk_n * 16);
    back(out->G_lesser, pb.Gl, blk_n * 16);
    back(out->G_greater, pb.Gg, blk_n * 16);
    back(out->Jdens, pb.Jd, blk_n * 16);
    back(out->bond_cur, pb.bond, npts * (nx - 1) * 8);
    back(out->status, pb.status, npts * 4);
    back(out->sancho_iters, pb.iters, npts * 8);
    flags |= QT_FLAG_SYNC;
  }
  if (flags & QT_FLAG_SYNC) {
    QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (out->status) {
      std::vector<int> hs;
      const int* st_h = out->status;
      if (devp) {
        hs.resize(npts);
        cudaMemcpy(hs.data(), out->status, npts * sizeof(int), cudaMemcpyDeviceToHost);
        st_h = hs.data();
      }
      for (long long p = 0; p < npts; ++p)
        if (st_h[p]) return QT_ERR_POINTS;
    }
  }
  return QT_OK;
}

extern "C" qt_status qt_rgf_solve_vb(qt_ctx* ctx, const qt_device_vb* dev, const double* E,
                                     int nE, const qt_contacts* c, qt_precision prec,
                                     unsigned flags, qt_outputs* out) {
  if (!ctx || !dev || !E || !c || !out) QT_FAIL(QT_ERR_ARG, "null argument");
  if (dev->nx < 2 || dev->nk <= 0 || nE <= 0 || !dev->nm || !dev->hii_off || !dev->h1i_off)
    QT_FAIL(QT_ERR_ARG, "need nx >= 2, nk > 0, nE > 0 and the block tables");
  if (!dev->Hii || !dev->H1i) QT_FAIL(QT_ERR_ARG, "Hii/H1i required");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (c->sancho_max_iter <= 0) QT_FAIL(QT_ERR_ARG, "sancho_max_iter must be > 0");
  if (c->quirks & QT_QUIRK_GLP_ZERO) QT_FAIL(QT_ERR_UNSUPPORTED, "QT_QUIRK_GLP_ZERO needs equal blocks");
  if (out->G_r || out->G_lesser || out->G_greater || out->Jdens)
    QT_FAIL(QT_ERR_UNSUPPORTED, "variable blocks: diagonal outputs and bond currents only");
  cudaSetDevice(ctx->device);
  ProblemVB pb{};
  pb.nx = dev->nx; pb.nk = dev->nk;
  pb.npts = (long long)nE * dev->nk;
  pb.c = *c; pb.prec = prec; pb.flags = flags;
  pb.hk = dev->hii_kstride; pb.h1k = dev->h1i_kstride;
  long long hii_n = 0, h1i_n = 0;
  for (int l = 0; l < dev->nx; ++l) {
    const int nl = dev->nm[l];
    if (nl <= 0) QT_FAIL(QT_ERR_ARG, "block sizes must be > 0");
    pb.n.push_back(nl);
    pb.nmax = std::max(pb.nmax, nl);
    pb.hoff.push_back(dev->hii_off[l]);
    pb.doff.push_back(pb.dsum);
    pb.dsum += nl;
    pb.goff.push_back(pb.gsum);
    pb.gsum += (long long)nl * nl;
    hii_n = std::max(hii_n, (long long)dev->hii_off[l] + (long long)nl * nl);
  }
  for (int l = 0; l <= dev->nx; ++l) {
    const int rows = l == 0 ? pb.n[0] : (l == dev->nx ? pb.n[dev->nx - 1] : pb.n[l]);
    const int cols = l == 0 ? pb.n[0] : (l == dev->nx ? pb.n[dev->nx - 1] : pb.n[l - 1]);
    pb.h1off.push_back(dev->h1i_off[l]);
    h1i_n = std::max(h1i_n, (long long)dev->h1i_off[l] + (long long)rows * cols);
  }
  if (prec != QT_PREC_FP64 && pb.nmax > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "split-precision path needs blocks <= 384");
  hii_n += pb.hk ? (dev->nk - 1) * pb.hk : 0;
  h1i_n += pb.h1k ? (dev->nk - 1) * pb.h1k : 0;
  const long long npts = pb.npts, diag_n = npts * pb.dsum;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  if (devp) {
    pb.Hii = reinterpret_cast<const cd*>(dev->Hii);
    pb.H1i = reinterpret_cast<const cd*>(dev->H1i);
    pb.E = E;
    pb.tr = out->tr; pb.tre = out->tre; pb.T = out->T;
    pb.dgr = out->diag_gr; pb.dgl = out->diag_gl; pb.dgg = out->diag_gg;
    pb.bond = out->bond_cur;
    pb.status = out->status; pb.iters = out->sancho_iters;
    QT_TRY(run_problem_vb(ctx, pb, hii_n, h1i_n));
  } else {
    size_t need = 0;
    auto add = [&](size_t bytes) { need += (bytes + 255) & ~size_t(255); };
    add(hii_n * 16); add(h1i_n * 16); add(nE * 8);
    add(npts * 8 * 3); add(diag_n * 16 * 3); add(npts * 4 * 3);
    if (out->bond_cur) add(npts * (pb.nx - 1) * 8);
    QT_TRY(ensure(ctx->io, ctx->io_bytes, need + 4096));
    HostStage st{ctx, reinterpret_cast<char*>(ctx->io)};
    pb.Hii = st.put(reinterpret_cast<const cd*>(dev->Hii), hii_n, true);
    pb.H1i = st.put(reinterpret_cast<const cd*>(dev->H1i), h1i_n, true);
    pb.E = st.put(E, nE, true);
    pb.tr = out->tr ? st.put<double>(nullptr, npts, false) : nullptr;
    pb.tre = out->tre ? st.put<double>(nullptr, npts, false) : nullptr;
    pb.T = out->T ? st.put<double>(nullptr, npts, false) : nullptr;
    pb.dgr = out->diag_gr ? st.put<double>(nullptr, 2 * diag_n, false) : nullptr;
    pb.dgl = out->diag_gl ? st.put<double>(nullptr, 2 * diag_n, false) : nullptr;
    pb.dgg = out->diag_gg ? st.put<double>(nullptr, 2 * diag_n, false) : nullptr;
    pb.bond = out->bond_cur ? st.put<double>(nullptr, npts * (pb.nx - 1), false) : nullptr;
    pb.status = st.put<int>(nullptr, npts, false);
    pb.iters = st.put<int>(nullptr, 2 * npts, false);
    QT_TRY(run_problem_vb(ctx, pb, hii_n, h1i_n));
    auto back = [&](void* dst, const void* src, size_t bytes) {
      if (dst && src) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    };
    back(out->tr, pb.tr, npts * 8);
    back(out->tre, pb.tre, npts * 8);
    back(out->T, pb.T, npts * 8);
    back(out->diag_gr, pb.dgr, diag_n * 16);
    back(out->diag_gl, pb.dgl, diag_n * 16);
    back(out->diag_gg, pb.dgg, diag_n * 16);
    back(out->bond_cur, pb.bond, npts * (pb.nx - 1) * 8);
    back(out->status, pb.status, npts * 4);
    back(out->sancho_iters, pb.iters, npts * 8);
    flags |= QT_FLAG_SYNC;
  }
  if (flags & QT_FLAG_SYNC) {
    QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (out->status) {
      std::vector<int> hs(npts);
      cudaMemcpy(hs.data(), out->status, npts * sizeof(int),
                 devp ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost);
      for (long long p = 0; p < npts; ++p)
        if (hs[p]) return QT_ERR_POINTS;
    }
  }
  return QT_OK;
}

extern "C" qt_status qt_rgf_constblocksize(qt_ctx* ctx, int nm, int nx, double En, double mul,
                                           double mur, double templ, double tempr,
                                           const double* Hii, const double* H1i, const double* Sii,
                                           const double* sigma_lesser_ph, const double* sigma_r_ph,
                                           double* G_r, double* G_lesser, double* G_greater,
                                           double* Jdens, double* tr, double* tre) {
  if (Sii) {
    // S = I is the only overlap the reference drivers build (src/deviceHam_mod.f90:281-284);
    // accept an explicit identity, reject anything else.
    for (int j = 0; j < nx; ++j)
      for (int c = 0; c < nm; ++c)
        for (int r = 0; r < nm; ++r) {
          const double* v = Sii + 2 * ((long long)j * nm * nm + (long long)c * nm + r);
          if (v[0] != (r == c ? 1.0 : 0.0) || v[1] != 0.0)
            QT_FAIL(QT_ERR_UNSUPPORTED, "Sii must be the identity");
        }
  }
  qt_device dev{};
  dev.nm = nm; dev.nx = nx; dev.nk = 1;
  dev.Hii = Hii; dev.hii_kstride = 0; dev.hii_lstride = (int64_t)nm * nm;
  dev.H1i = H1i; dev.h1i_kstride = 0; dev.h1i_lstride = (int64_t)nm * nm;
  qt_contacts c{};
  c.mul = mul; c.mur = mur; c.templ = templ; c.tempr = tempr;
  c.eta_lead = 1e-5; c.eta_interior = 0.0; c.sancho_tol = 1e-100; c.sancho_max_iter = 50;
  c.quirks = 0;
  qt_outputs o{};
  o.tr = tr; o.tre = tre; o.G_r = G_r; o.G_lesser = G_lesser; o.G_greater = G_greater;
  o.Jdens = Jdens;
  return qt_rgf_solve(ctx, &dev, &En, 1, &c, sigma_r_ph, sigma_lesser_ph, QT_PREC_FP64, 0, &o);
}

extern "C" qt_status qt_sancho_batch(qt_ctx* ctx, int nm, int npts, const double* E,
                                     const double* H00, int64_t h00_stride, const double* H10,
                                     int64_t h10_stride, const double* S00, int64_t s00_stride,
                                     double eta, double tol, int max_iter, qt_precision prec,
                                     unsigned flags, double* G00, double* GBB, int* iters,
                                     int* status) {
  (void)s00_stride;
  if (!ctx || !E || !H00 || !H10 || !G00 || nm <= 0 || npts <= 0 || max_iter <= 0)
    QT_FAIL(QT_ERR_ARG, "bad sancho arguments");
  if (S00) QT_FAIL(QT_ERR_UNSUPPORTED, "S00 must be NULL (identity overlap)");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec == QT_PREC_MIXED_FP64) prec = QT_PREC_MIXED;  // blocks are complex128 in both
  if (prec == QT_PREC_MIXED && nm > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "split-precision path needs nm <= 384");
  cudaSetDevice(ctx->device);
  const long long nm2 = (long long)nm * nm;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  const long long P = npts;
  // scratch: z, status, iters, 2 refinement blocks + Sancho state (7 blocks)
  const size_t need = (size_t)P * nm2 * sizeof(cd) * (9 + (devp ? 0 : 2)) + (size_t)P * 64 +
                      (h00_stride ? P : 1) * nm2 * 16 + (h10_stride ? P : 1) * nm2 * 16 +
                      (size_t)P * 1100 + (1 << 20);
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, need));
  Arena ar{reinterpret_cast<char*>(ctx->arena), ctx->arena_bytes, 0};
  cudaStream_t s = ctx->stream;
  Ops<double2> op{s, nm, prec};
  op.slices = env_int("QT_LEAD_SLICES", 7);
  op.refine = prec == QT_PREC_FP64 ? 0 : 3;
  cd* one = ar.take<cd>(1);
  const cd h1{1.0, 0.0};
  cudaMemcpyAsync(one, &h1, sizeof(cd), cudaMemcpyHostToDevice, s);
  op.one = one;
  cd* z = ar.take<cd>(P);
  int* st = ar.take<int>(P);
  int* it = ar.take<int>(P);
  const double* Ed = E;
  const cd *h00 = reinterpret_cast<const cd*>(H00), *h10 = reinterpret_cast<const cd*>(H10);
  cd *g00 = reinterpret_cast<cd*>(G00), *gbb = reinterpret_cast<cd*>(GBB);
  if (!devp) {
    double* e = ar.take<double>(P);
    cudaMemcpyAsync(e, E, P * 8, cudaMemcpyHostToDevice, s);
    Ed = e;
    cd* a = ar.take<cd>((h00_stride ? P : 1) * nm2);
    cudaMemcpyAsync(a, H00, (h00_stride ? P : 1) * nm2 * 16, cudaMemcpyHostToDevice, s);
    h00 = a;
    cd* b = ar.take<cd>((h10_stride ? P : 1) * nm2);
    cudaMemcpyAsync(b, H10, (h10_stride ? P : 1) * nm2 * 16, cudaMemcpyHostToDevice, s);
    h10 = b;
    g00 = ar.take<cd>(P * nm2);
    gbb = GBB ? ar.take<cd>(P * nm2) : nullptr;
  }
  if (!one || !z || !st || !it || !g00) QT_FAIL(QT_ERR_NOMEM, "arena exhausted");
  make_z_kernel<<<g1d(P), 256, 0, s>>>(Ed, 0, P, 1, eta, z);
  qt::count_launch();
  cudaMemsetAsync(st, 0, P * 4, s);
  QT_TRY(sancho_wave(op, ar, P, ref(h00, h00_stride ? nm2 : 0, nm), ref(h10, h10_stride ? nm2 : 0, nm),
                     false, z, tol, max_iter, ref(g00, nm2, nm), gbb ? ref(gbb, nm2, nm) : nullref(),
                     st, it, 1, nullref(), (flags & QT_FLAG_SANCHO_RESET) != 0));
  if (prec != QT_PREC_FP64) {
    QT_CUDA_TRY(cudaStreamSynchronize(s));
    if (qt::oz_timeouts_and_reset()) QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  }
  if (!devp) {
    cudaMemcpyAsync(G00, g00, P * nm2 * 16, cudaMemcpyDeviceToHost, s);
    if (GBB) cudaMemcpyAsync(GBB, gbb, P * nm2 * 16, cudaMemcpyDeviceToHost, s);
    if (iters) cudaMemcpyAsync(iters, it, P * 4, cudaMemcpyDeviceToHost, s);
    if (status) cudaMemcpyAsync(status, st, P * 4, cudaMemcpyDeviceToHost, s);
  } else {
    if (iters) cudaMemcpyAsync(iters, it, P * 4, cudaMemcpyDeviceToDevice, s);
    if (status) cudaMemcpyAsync(status, st, P * 4, cudaMemcpyDeviceToDevice, s);
  }
  QT_CUDA_TRY(cudaStreamSynchronize(s));
  return QT_OK;
}

namespace {
int parse_op(char c) {
  if (c == 'N' || c == 'n') return qt::OP_N;
  if (c == 'C' || c == 'c') return qt::OP_C;
  if (c == 'T' || c == 't') return qt::OP_T;
  return -1;
}
}  // namespace

extern "C" qt_status qt_zgemm_batch(qt_ctx* ctx, int n, int batch, char opA, const double* A,
                                    int64_t a_stride, char opB, const double* B, int64_t b_stride,
                                    const double* alpha, const double* beta, const double* D,
                                    int64_t d_stride, double* C, int64_t c_stride,
                                    qt_precision prec, int slices, unsigned flags) {
  const int oa = parse_op(opA), ob = parse_op(opB);
  if (!ctx || !A || !B || !C || n <= 0 || batch <= 0 || oa < 0 || ob < 0)
    QT_FAIL(QT_ERR_ARG, "bad gemm arguments");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec == QT_PREC_MIXED_FP64) prec = QT_PREC_MIXED;  // blocks are complex128 in both
  if (prec == QT_PREC_MIXED && (n > MAX_SPLIT || oa == qt::OP_T || ob == qt::OP_T))
    QT_FAIL(QT_ERR_UNSUPPORTED, "mixed gemm: n <= 384 and op in {N, C}");
  if (slices < 0 || slices > 8) QT_FAIL(QT_ERR_ARG, "slices in 0..8");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const long long nm2 = (long long)n * n;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  const cd al = alpha ? cd{alpha[0], alpha[1]} : cd{1, 0};
  const cd be = beta ? cd{beta[0], beta[1]} : cd{0, 0};
  if (flags & QT_FLAG_COMPLEX64) {
    // complex64 blocks (the complex64 sweep's 4-digit split product), device pointers
    if (!devp || prec != QT_PREC_MIXED || (slices != 0 && slices != 4) || al.y != 0.0 ||
        be.y != 0.0)
      QT_FAIL(QT_ERR_UNSUPPORTED,
              "complex64 product: device pointers, QT_PREC_MIXED, 4 digits, real alpha/beta");
    QT_TRY(ensure(ctx->arena, ctx->arena_bytes, (size_t)batch * 1024 + 4096));
    Ops<float2> op{s, n, prec};
    op.slices = 4;
    op.scales = reinterpret_cast<int*>(ctx->arena);
    op.P = batch;
    op.prof = &ctx->prof;
    QT_TRY(op.gemm3(n, n, n, ref(A, a_stride, n), oa, ref(B, b_stride, n), ob,
                    ref(C, c_stride, n), batch, al, D ? ref(D, d_stride, n) : nullref(), be));
    if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(s));
    return QT_OK;
  }
  const void *a = A, *b = B, *d = D;
  void* c = C;
  if (!devp) {
    auto cnt = [&](int64_t st) { return (long long)(st ? (long long)(batch - 1) * st + nm2 : nm2); };
    size_t need = (cnt(a_stride) + cnt(b_stride) + (D ? cnt(d_stride) : 0) + cnt(c_stride)) * 16 + 4096;
    QT_TRY(ensure(ctx->io, ctx->io_bytes, need));
    HostStage hs{ctx, reinterpret_cast<char*>(ctx->io)};
    a = hs.put(reinterpret_cast<const cd*>(A), cnt(a_stride), true);
    b = hs.put(reinterpret_cast<const cd*>(B), cnt(b_stride), true);
    d = D ? hs.put(reinterpret_cast<const cd*>(D), cnt(d_stride), true) : nullptr;
    c = hs.put<cd>(nullptr, cnt(c_stride), false);
  }
  qt::GemmArgs g;
  g.m = g.n = g.k = n;
  g.A = ref(a, a_stride, n); g.B = ref(b, b_stride, n); g.C = ref(c, c_stride, n);
  g.D = d ? ref(d, d_stride, n) : nullref(); g.Z = nullref();
  g.opA = oa; g.opB = ob;
  g.alpha_re = al.x; g.alpha_im = al.y; g.beta_re = be.x; g.beta_im = be.y;
  g.batch = batch; g.active = nullptr;
  g.scales = nullptr;
  const int sl = slices ? slices : 4;
  if (prec == QT_PREC_MIXED && sl != 4 && sl != 6 && sl != 7)
    QT_FAIL(QT_ERR_UNSUPPORTED, "complex128 split product supports 4, 6 or 7 digits");
  if (prec == QT_PREC_FP64) {
    cudaError_t e = qt::zgemm_f64(g, s);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  } else {
    // through the block operations, which tile blocks above one 128-row tile
    QT_TRY(ensure(ctx->arena, ctx->arena_bytes, (size_t)batch * 1024 + 4096));
    Ops<double2> op{s, n, prec};
    op.slices = sl;
    op.scales = reinterpret_cast<int*>(ctx->arena);
    op.P = batch;
    op.prof = &ctx->prof;
    QT_TRY(op.gemm3(n, n, n, g.A, oa, g.B, ob, g.C, batch, al, g.D, be));
  }
  if (!devp) {
    const long long cc = c_stride ? (long long)(batch - 1) * c_stride + nm2 : nm2;
    cudaMemcpyAsync(C, c, cc * 16, cudaMemcpyDeviceToHost, s);
  }
  if (!devp || (flags & QT_FLAG_SYNC)) QT_CUDA_TRY(cudaStreamSynchronize(s));
  return QT_OK;
}

extern "C" qt_status qt_zinv_batch(qt_ctx* ctx, int n, int batch, const double* A,
                                   int64_t a_stride, double* X, int64_t x_stride,
                                   qt_precision prec, unsigned flags, int* status) {
  if (!ctx || !A || !X || n <= 0 || batch <= 0) QT_FAIL(QT_ERR_ARG, "bad inverse arguments");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec == QT_PREC_MIXED_FP64) prec = QT_PREC_MIXED;  // blocks are complex128 in both
  if (prec == QT_PREC_MIXED && n > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "mixed inverse needs n <= 384");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const long long nm2 = (long long)n * n;
  const bool devp = (flags & QT_FLAG_DEVICE_POINTERS) != 0;
  const long long P = batch;
  const size_t need = (size_t)P * nm2 * 16 * (3 + (devp ? 0 : 2)) + (size_t)P * 1400 + (1 << 20);
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, need));
  Arena ar{reinterpret_cast<char*>(ctx->arena), ctx->arena_bytes, 0};
  Ops<double2> op{s, n, prec};
  op.guard = ar.take<unsigned char>(P);
  op.fallbacks = ctx->fallbacks;
  op.P = P;
  op.slices = env_int("QT_LEAD_SLICES", 7);
  op.refine = prec == QT_PREC_FP64 ? 0 : 3;
  cd* one = ar.take<cd>(1);
  const cd h1{1.0, 0.0};
  cudaMemcpyAsync(one, &h1, sizeof(cd), cudaMemcpyHostToDevice, s);
  op.one = one;
  op.rt1 = reinterpret_cast<double2*>(ar.take<cd>(P * nm2));
  op.rt2 = reinterpret_cast<double2*>(ar.take<cd>(P * nm2));
  op.scales = ar.take<int>(P * 256);
  int* st = ar.take<int>(P);
  const cd* a = reinterpret_cast<const cd*>(A);
  cd* x = reinterpret_cast<cd*>(X);
  long long as = a_stride, xs = x_stride;
  if (!devp) {
    cd* ad = ar.take<cd>(P * nm2);
    cd* xd = ar.take<cd>(P * nm2);
    if (!ad || !xd) QT_FAIL(QT_ERR_NOMEM, "arena exhausted");
    for (long long b = 0; b < P; ++b)
      cudaMemcpyAsync(ad + b * nm2, reinterpret_cast<const cd*>(A) + b * a_stride, nm2 * 16,
                      cudaMemcpyHostToDevice, s);
    a = ad; x = xd; as = nm2; xs = nm2;
  } else if (prec == QT_PREC_MIXED && (const void*)A == (const void*)X) {
    cd* ad = ar.take<cd>(P * nm2);
    if (!ad) QT_FAIL(QT_ERR_NOMEM, "arena exhausted");
    cudaMemcpyAsync(ad, A, P * nm2 * 16, cudaMemcpyDeviceToDevice, s);
    a = ad; as = nm2;
  }
  if (!st || !op.rt2 || !op.scales) QT_FAIL(QT_ERR_NOMEM, "arena exhausted");
  cudaMemsetAsync(st, 0, P * 4, s);
  QT_TRY(op.inv(ref(a, as, n), ref(x, xs, n), P, st));
  if (!devp) {
    for (long long b = 0; b < P; ++b)
      cudaMemcpyAsync(X + 2 * b * x_stride, x + b * nm2, nm2 * 16, cudaMemcpyDeviceToHost, s);
    if (status) cudaMemcpyAsync(status, st, P * 4, cudaMemcpyDeviceToHost, s);
  } else if (status) {
    cudaMemcpyAsync(status, st, P * 4, cudaMemcpyDeviceToDevice, s);
  }
  QT_CUDA_TRY(cudaStreamSynchronize(s));
  return QT_OK;
}

// ================================================================ GW / SCBA
// One evaluation of the SCBA map Sigma -> Sigma_new (gw_ephoton_3d_ijs,
// src/gw_mod.f90:368-749): G by the batched RGF with the scattering self-energies at
// every k-point (green_RGF_RS, :1131-1345), P by energy correlations of the Re-zeroed G
// summed over k-pairs (:444-519), W per momentum transfer and slab-diagonal block
// (green_rgf_calc_w is absent from the reference; restated as
// W^R = (I - V_q P^R)^-1 V_q, W^{<,>} = W^R P^{<,>} W^R^+), Sigma by energy
// convolutions summed over k-pairs (:646-698), the ndiag band of P and Sigma
// (:471-475, 527-555, 705-730), recombination + symmetrisation (:698, 731-743) and
// the edge-block copy (:950-959).
namespace {

// k-point grid and band of one GW problem
struct GwGrid {
  int nk = 1, nky = 1, nkz = 1, ndiag = -1;
  bool v_per_slab = false;  // V holds [nk][nx] blocks (QT_FLAG_V_PER_SLAB)
  long long hk = 0, h1k = 0;  // H / H1i strides between k-points (complex elements)
};

// The map holds six [nk][nE][nx][nm^2] arrays: G^{R,<,>}, then P^{R,<,>}, which become
// W^{R,<,>} in place.  With one k-point the new self-energies are written over G (a
// series is read completely before it is written), so NR/NL/NG alias GR/GL/GG; the
// k-pair sums read every k of G, so with several k-points they have arrays of their own.
struct GwBuffers {
  cd *GR, *GL, *GG, *PR, *PL, *PG, *NR, *NL, *NG;
  double2* tw;
  double* sums;
};

// Optional per-energy currents of the map's RGF (green_RGF_RS's tr, tre, cur): device [nE],
// [nE], [nE][nx-1]
struct GwCurrents {
  double *tr = nullptr, *tre = nullptr, *bond = nullptr;
};

// W^R = (I - V P^R)^-1 V and W^{<,>} = W^R P^{<,>} W^R^+ per (w, slab) block, nblk blocks of
// nm x nm at stride bstride (0: nm^2), in chunks of blocks whose scratch (two chunk-sized
// blocks, the refinement blocks, exponent table and guard flags) comes from the context
// arena.  Each output may alias its own P (W^R -> P^R, W^< -> P^<, W^> -> P^>): a chunk of
// P is read before that chunk of W is written.
qt_status gw_screened_blocks(qt_ctx* ctx, int nm, long long nblk, qt_precision prec,
                             int slices, const cd* V, const cd* PR, const cd* PL, const cd* PG,
                             cd* WR, cd* WL, cd* WG, int ndiag = -1, long long bstride = 0) {
  cudaStream_t s = ctx->stream;
  const long long nm2 = (long long)nm * nm;
  Ops<double2> op{s, nm, prec};
  op.slices = slices;
  op.refine = prec == QT_PREC_FP64 ? 0 : 2;
  op.prof = &ctx->prof;
  // about 8 GB of scratch per chunk
  const size_t per_block = 4 * (size_t)nm2 * 16 + 1300;
  const long long chunk = std::max(1LL, std::min(nblk, (long long)((8ull << 30) / per_block)));
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, (size_t)chunk * per_block + 8192));
  Arena ar{reinterpret_cast<char*>(ctx->arena), ctx->arena_bytes, 0};
  cd* one = ar.take<cd>(1);
  const cd h1{1.0, 0.0};
  cudaMemcpyAsync(one, &h1, sizeof(cd), cudaMemcpyHostToDevice, s);
  op.one = one;
  op.scales = ar.take<int>((size_t)chunk * 256);
  op.rt1 = reinterpret_cast<double2*>(ar.take<cd>((size_t)chunk * nm2));
  op.rt2 = reinterpret_cast<double2*>(ar.take<cd>((size_t)chunk * nm2));
  op.P = chunk;
  op.guard = ar.take<unsigned char>((size_t)chunk);
  op.fallbacks = ctx->fallbacks;
  cd* T1 = ar.take<cd>((size_t)chunk * nm2);
  cd* T2 = ar.take<cd>((size_t)chunk * nm2);
  if (!op.scales || !op.rt2 || !op.guard || !T1 || !T2)
    QT_FAIL(QT_ERR_NOMEM, "arena exhausted (W)");
  if (!bstride) bstride = nm2;
  const BatchRef Vr = ref(V, 0, nm), B = ref(nullptr, nm2, nm), Bs = ref(nullptr, bstride, nm);
  auto blk = [&](const cd* p) { BatchRef r = B; r.p = const_cast<cd*>(p); return r; };  // scratch
  auto arr = [&](const cd* p) { BatchRef r = Bs; r.p = const_cast<cd*>(p); return r; };  // P, W
  // the ndiag band of P (src/gw_mod.f90:527-555): a banded copy of each P chunk (in T2
  // for P^R, in the W chunk for P^< and P^>, which the products below then overwrite)
  auto banded = [&](BatchRef P, BatchRef dst, long long cb) -> bool {
    qt::zcopy<double2>(nm, cb, P, dst, s);
    return qt::gw_band_zero(nm, cb, ndiag, reinterpret_cast<double2*>(dst.p), s,
                            dst.stride) == cudaSuccess;
  };
  for (long long c0 = 0; c0 < nblk; c0 += chunk) {
    const long long cb = std::min(chunk, nblk - c0), o = c0 * bstride;
    // T1 = I - V P^R ; T2 = T1^-1 ; T1 = T2 V = W^R
    BatchRef pr = arr(PR + o), pl = arr(PL + o), pg = arr(PG + o);
    if (ndiag >= 0) {
      if (!banded(pr, blk(T2), cb)) QT_FAIL(QT_ERR_CUDA, "band launch failed");
      pr = blk(T2);
    }
    QT_TRY(op.gemm(Vr, qt::OP_N, pr, qt::OP_N, blk(T1), cb, {-1, 0}, nullref(), {0, 0},
                   ref(one, 0, 1)));
    QT_TRY(op.inv(blk(T1), blk(T2), cb, nullptr));
    QT_TRY(op.gemm(blk(T2), qt::OP_N, Vr, qt::OP_N, blk(T1), cb));
    // W^< = W^R P^< W^R^+, W^> = W^R P^> W^R^+ (a banded P^< / P^> goes to its W chunk first)
    if (ndiag >= 0) {
      if (!banded(pl, arr(WL + o), cb)) QT_FAIL(QT_ERR_CUDA, "band launch failed");
      pl = arr(WL + o);
    }
    QT_TRY(op.gemm(blk(T1), qt::OP_N, pl, qt::OP_N, blk(T2), cb));
    QT_TRY(op.gemm(blk(T2), qt::OP_N, blk(T1), qt::OP_C, arr(WL + o), cb));
    if (ndiag >= 0) {
      if (!banded(pg, arr(WG + o), cb)) QT_FAIL(QT_ERR_CUDA, "band launch failed");
      pg = arr(WG + o);
    }
    QT_TRY(op.gemm(blk(T1), qt::OP_N, pg, qt::OP_N, blk(T2), cb));
    QT_TRY(op.gemm(blk(T2), qt::OP_N, blk(T1), qt::OP_C, arr(WG + o), cb));
    qt::zcopy<double2>(nm, cb, blk(T1), arr(WR + o), s);
  }
  return QT_OK;
}

// The ndiag band (src/gw_mod.f90:705-730), Sigma^R <- Re Sigma^R + i Im(Sigma^> -
// Sigma^<)/2, (S + S^T)/2 (:698, 731-743) and the edge blocks 1,2 <- 3 and nx-1,nx <- nx-2
// (:950-959) for nE energies (all k-points) of nx slab blocks
qt_status gw_post(qt_ctx* ctx, int nm, int nx, long long nE, cd* NR, cd* NL, cd* NG,
                  int ndiag = -1) {
  cudaStream_t s = ctx->stream;
  const long long nm2 = (long long)nm * nm;
  if (ndiag >= 0)
    for (cd* S : {NR, NL, NG}) {
      cudaError_t e = qt::gw_band_zero(nm, nE * nx, ndiag, reinterpret_cast<double2*>(S), s);
      if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    }
  cudaError_t e = qt::gw_sigma_post(nm, nE * nx, reinterpret_cast<double2*>(NR),
                                    reinterpret_cast<double2*>(NL),
                                    reinterpret_cast<double2*>(NG), s);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  if (nx >= 5) {
    for (cd* S : {NR, NL, NG}) {
      auto slab = [&](int l) { return ref(S + l * nm2, nx * nm2, nm); };
      qt::zcopy<double2>(nm, nE, slab(2), slab(0), s);
      qt::zcopy<double2>(nm, nE, slab(2), slab(1), s);
      qt::zcopy<double2>(nm, nE, slab(nx - 3), slab(nx - 1), s);
      qt::zcopy<double2>(nm, nE, slab(nx - 3), slab(nx - 2), s);
    }
  }
  return QT_OK;
}

qt_status gw_map(qt_ctx* ctx, Problem pb, const GwGrid& g, const cd* V, double spindeg,
                 const cd* SR, const cd* SL, GwBuffers& w, long long hii_n, long long h1i_n,
                 const GwCurrents& cur = GwCurrents{}) {
  cudaStream_t s = ctx->stream;
  const int nm = pb.nm, nx = pb.nx, nk = g.nk;
  const long long nE = pb.npts;  // energies per k-point
  const long long nm2 = (long long)nm * nm, nblk = nE * nx, kst = nblk * nm2;
  // digits of the screened interaction's products: the leads' FP64 grade, as run_problem
  // sets them for the RGF
  pb.lead_slices = env_int("QT_LEAD_SLICES", 7);
  // ---- G with the current self-energies, one k-point at a time (its H blocks)
  const cd* Hii = pb.Hii;
  const cd* H1i = pb.H1i;
  ProfPhase ph_rgf(ctx->prof, s, 5);
  for (int k = 0; k < nk; ++k) {
    Problem pk = pb;
    pk.Hii = Hii + k * g.hk;
    pk.H1i = H1i + k * g.h1k;
    pk.sigr = SR + k * kst;
    pk.sigl = SL + k * kst;
    pk.T = pk.dgr = pk.dgl = pk.dgg = nullptr;
    pk.tr = cur.tr ? cur.tr + k * nE : nullptr;
    pk.tre = cur.tre ? cur.tre + k * nE : nullptr;
    pk.bond = cur.bond ? cur.bond + k * nE * (nx - 1) : nullptr;
    pk.Jd = nullptr;
    pk.Gr = w.GR + k * kst; pk.Gl = w.GL + k * kst; pk.Gg = w.GG + k * kst;
    pk.flags &= ~QT_FLAG_CAROLI;
    QT_TRY(run_problem(ctx, pk, hii_n, h1i_n));
  }
  ph_rgf.end();
  // ---- polarisation: energy correlations of Re-zeroed G, x -i dE/(2 pi) spindeg / nk
  double dE = 0.0;
  {
    double e2[2] = {0, 0};
    cudaMemcpyAsync(e2, pb.E, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    QT_CUDA_TRY(cudaStreamSynchronize(s));
    dE = e2[1] - e2[0];
  }
  const double pf = dE / (2.0 * M_PI) * spindeg / nk;  // P scale = -i * pf
  qt::CorrConvArgs c{};
  c.n = (int)nE; c.nm = nm; c.nseries = nx * nm2; c.estride = nx * nm2;
  c.nk = nk; c.nky = g.nky; c.nkz = g.nkz; c.kstride = kst; c.ndiag = g.ndiag;
  auto run = [&](const qt::CorrConvArgs& a) -> qt_status {
    cudaError_t e = qt::zcorrconv(a, w.tw, s);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    return QT_OK;
  };
  auto cc = [&](const cd* X, const cd* Y, cd* Z, int corr, int transY, int conjY, int imX,
                int imY, double sr, double si, int kmode) -> qt_status {
    qt::CorrConvArgs a = c;
    a.X = X; a.Y = Y; a.Z = Z; a.corr = corr; a.transY = transY; a.conjY = conjY;
    a.imagX = imX; a.imagY = imY; a.scale_re = sr; a.scale_im = si; a.kmode = kmode;
    return run(a);
  };
  // one k-point: all three P from packed transforms of the imaginary G in one launch
  qt::GwFusedArgs pk{};
  pk.n = (int)nE; pk.nm = nm; pk.nseries = nx * nm2; pk.estride = nx * nm2;
  pk.ndiag = g.ndiag;
  ProfPhase ph_pol(ctx->prof, s, 6);
  if (nk == 1) {
    qt::GwFusedArgs a = pk;
    a.GR = w.GR; a.GL = w.GL; a.GG = w.GG;  // transposed partners: element (j, i)
    a.PR = w.PR; a.PL = w.PL; a.PG = w.PG;
    a.scale_re = 0.0; a.scale_im = -pf;
    cudaError_t e = qt::gw_polarization_packed(a, w.tw, s);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  } else {
    QT_TRY(cc(w.GL, w.GG, w.PL, 1, 1, 0, 1, 1, 0.0, -pf, 1));  // P^< = corr(G^<_ij, G^>_ji)
    QT_TRY(cc(w.GG, w.GL, w.PG, 1, 1, 0, 1, 1, 0.0, -pf, 1));  // P^> = corr(G^>_ij, G^<_ji)
    // P^R = corr(G^<_ij, conj G^R_ij) + corr(G^R_ij, G^<_ji), one inverse transform
    qt::CorrConvArgs a = c;
    a.X = w.GL; a.Y = w.GR; a.conjY = 1; a.X2 = w.GR; a.Y2 = w.GL; a.transY2 = 1;
    a.Z = w.PR; a.corr = 1; a.imagX = 1; a.imagY = 1; a.scale_re = 0.0; a.scale_im = -pf;
    a.kmode = 1;
    QT_TRY(run(a));
  }
  ph_pol.end();
  // ---- screened interaction per momentum transfer q and (w, slab) block, in place: P -> W;
  // with a Coulomb block per slab, the blocks of slab x (every energy) take V_{q,x}
  ProfPhase ph_w(ctx->prof, s, 7);
  for (int q = 0; q < nk; ++q) {
    const long long o = q * kst;
    if (!g.v_per_slab) {
      QT_TRY(gw_screened_blocks(ctx, nm, nblk, pb.prec, pb.lead_slices, V + q * nm2, w.PR + o,
                                w.PL + o, w.PG + o, w.PR + o, w.PL + o, w.PG + o, g.ndiag));
      continue;
    }
    for (int x = 0; x < nx; ++x) {
      const long long ox = o + x * nm2;
      QT_TRY(gw_screened_blocks(ctx, nm, nE, pb.prec, pb.lead_slices, V + (q * nx + x) * nm2,
                                w.PR + ox, w.PL + ox, w.PG + ox, w.PR + ox, w.PL + ox, w.PG + ox,
                                g.ndiag, nx * nm2));
    }
  }
  ph_w.end();
  // ---- self-energy: energy convolutions x i dE / (2 pi) / nk; with one k-point written
  // over G: Sigma^R first (it reads G^< and G^R), then Sigma^< over G^<, Sigma^> over G^>
  const double sf = dE / (2.0 * M_PI) / nk;
  ProfPhase ph_sig(ctx->prof, s, 6);
  if (nk == 1) {
    // Sigma^>, Sigma^<, Sigma^R of each series in one CTA, written over G
    qt::GwFusedArgs a = pk;
    a.GR = w.GR; a.GL = w.GL; a.GG = w.GG;
    a.WR = w.PR; a.WL = w.PL; a.WG = w.PG;
    a.SR = w.NR; a.SL = w.NL; a.SG = w.NG;
    a.scale_re = 0.0; a.scale_im = sf;
    cudaError_t e = qt::gw_selfenergy_packed(a, w.tw, s);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  } else {
    // Sigma^R = conv(G^<, W^R) + conv(G^R, W^<) + conv(G^R, W^R)
    //         = conv(G^<, W^R) + conv(G^R, W^< + W^R)
    qt::CorrConvArgs a = c;
    a.X = w.GL; a.Y = w.PR; a.X2 = w.GR; a.Y2 = w.PL; a.Y2b = w.PR;
    a.Z = w.NR; a.corr = 0; a.imagX = 1; a.scale_re = 0.0; a.scale_im = sf; a.kmode = 2;
    QT_TRY(run(a));
    QT_TRY(cc(w.GL, w.PL, w.NL, 0, 0, 0, 1, 0, 0.0, sf, 2));  // Sigma^< = conv(G^<, W^<)
    QT_TRY(cc(w.GG, w.PG, w.NG, 0, 0, 0, 1, 0, 0.0, sf, 2));  // Sigma^> = conv(G^>, W^>)
  }
  ph_sig.end();
  // ---- band, recombination, symmetrisation, edge blocks
  ProfPhase ph_post(ctx->prof, s, 8);
  QT_TRY(gw_post(ctx, nm, nx, nk * nE, w.NR, w.NL, w.NG, g.ndiag));
  return QT_OK;
}

qt_status gw_setup(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                   const qt_contacts* c, qt_precision prec, unsigned flags, Problem& pb,
                   GwGrid& g, long long& hii_n, long long& h1i_n) {
  if (!ctx || !dev || !E || !c) QT_FAIL(QT_ERR_ARG, "null argument");
  if (!(flags & QT_FLAG_DEVICE_POINTERS)) QT_FAIL(QT_ERR_UNSUPPORTED, "GW entry points take device pointers");
  if (dev->nk < 1) QT_FAIL(QT_ERR_ARG, "need nk >= 1");
  // the k-point grid: the context's when it covers dev->nk points, else one direction
  g = GwGrid{};
  g.nk = dev->nk;
  if (ctx->gw_nky * ctx->gw_nkz == dev->nk) {
    g.nky = ctx->gw_nky;
    g.nkz = ctx->gw_nkz;
  } else if (ctx->gw_nky * ctx->gw_nkz == 1) {
    g.nky = 1;
    g.nkz = dev->nk;
  } else {
    QT_FAIL(QT_ERR_ARG, "dev->nk differs from the k-point grid of qt_ctx_set_gw_grid");
  }
  g.ndiag = ctx->gw_ndiag;
  g.v_per_slab = (flags & QT_FLAG_V_PER_SLAB) != 0;
  g.hk = dev->hii_kstride;
  g.h1k = dev->h1i_kstride;
  if (dev->nk > 1 && (g.hk == 0 && g.h1k == 0))
    QT_FAIL(QT_ERR_ARG, "several k-points need H blocks per k (hii_kstride / h1i_kstride)");
  if (dev->nm <= 0 || dev->nx < 2 || nE < 2) QT_FAIL(QT_ERR_ARG, "need nm > 0, nx >= 2, nE >= 2");
  if (2 * nE > 4096) QT_FAIL(QT_ERR_UNSUPPORTED, "GW path: nE <= 2048 (FFT length 4096)");
  if (dev->Sii) QT_FAIL(QT_ERR_UNSUPPORTED, "Sii must be NULL (identity overlap)");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec != QT_PREC_FP64 && dev->nm > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "split-precision path needs nm <= 384");
  cudaSetDevice(ctx->device);
  pb = Problem{};  // one k-point per RGF call: gw_map offsets H by g.hk / g.h1k
  pb.nm = dev->nm; pb.nx = dev->nx; pb.nk = 1; pb.npts = nE;
  pb.Hii = reinterpret_cast<const cd*>(dev->Hii); pb.hk = 0; pb.hl = dev->hii_lstride;
  pb.H1i = reinterpret_cast<const cd*>(dev->H1i); pb.h1k = 0; pb.h1l = dev->h1i_lstride;
  pb.E = E; pb.c = *c; pb.prec = prec; pb.flags = flags;
  const long long nm2 = (long long)dev->nm * dev->nm;
  hii_n = (pb.hl ? (dev->nx - 1) * pb.hl : 0) + nm2;
  h1i_n = (pb.h1l ? dev->nx * pb.h1l : 0) + nm2;
  return QT_OK;
}

struct GwAlloc {
  void* p = nullptr;
  ~GwAlloc() { if (p) cudaFree(p); }
};

// cnt: elements of one [nk][nE][nx][nm^2] array; npts = nk * nE (per-point currents)
qt_status gw_alloc(qt_ctx* ctx, long long cnt, long long npts, int nk, GwBuffers& w,
                   GwAlloc& hold) {
  const size_t blk = (size_t)cnt * sizeof(cd);
  const int narr = nk > 1 ? 9 : 6;  // separate new self-energies for the k-pair sums
  // block arrays, FFT twiddles, then 64 B of sums and 2 x npts doubles of currents
  const size_t need = narr * blk + 2048 * sizeof(double2) + 64 + 2 * (size_t)npts * sizeof(double);
  if (cudaMalloc(&hold.p, need) != cudaSuccess) {
    cudaGetLastError();
    QT_FAIL(QT_ERR_NOMEM, "GW buffers");
  }
  char* b = reinterpret_cast<char*>(hold.p);
  cd** slots[] = {&w.GR, &w.GL, &w.GG, &w.PR, &w.PL, &w.PG, &w.NR, &w.NL, &w.NG};
  for (int i = 0; i < narr; ++i) *slots[i] = reinterpret_cast<cd*>(b + i * blk);
  if (narr == 6) {
    w.NR = w.GR;
    w.NL = w.GL;
    w.NG = w.GG;
  }
  w.tw = reinterpret_cast<double2*>(b + narr * blk);
  w.sums = reinterpret_cast<double*>(b + narr * blk + 2048 * sizeof(double2));
  cudaError_t e = qt::gw_twiddles(w.tw, ctx->stream);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

}  // namespace

extern "C" qt_status qt_gw_step(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                                const qt_contacts* c, const double* V, double spindeg,
                                qt_precision prec, unsigned flags, const double* sigma_r,
                                const double* sigma_lesser, double* new_r, double* new_lesser,
                                double* new_greater) {
  Problem pb;
  GwGrid g;
  long long hn, h1n;
  QT_TRY(gw_setup(ctx, dev, E, nE, c, prec, flags, pb, g, hn, h1n));
  if (!V || !sigma_r || !sigma_lesser || !new_r || !new_lesser || !new_greater)
    QT_FAIL(QT_ERR_ARG, "null GW array");
  const long long cnt = (long long)g.nk * nE * dev->nx * dev->nm * dev->nm;
  GwBuffers w{};
  GwAlloc hold;
  QT_TRY(gw_alloc(ctx, cnt, (long long)g.nk * nE, g.nk, w, hold));
  QT_TRY(gw_map(ctx, pb, g, reinterpret_cast<const cd*>(V), spindeg,
                reinterpret_cast<const cd*>(sigma_r), reinterpret_cast<const cd*>(sigma_lesser),
                w, hn, h1n));
  cudaStream_t s = ctx->stream;
  cudaMemcpyAsync(new_r, w.NR, cnt * 16, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(new_lesser, w.NL, cnt * 16, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(new_greater, w.NG, cnt * 16, cudaMemcpyDeviceToDevice, s);
  QT_CUDA_TRY(cudaStreamSynchronize(s));
  if (prec != QT_PREC_FP64 && qt::oz_timeouts_and_reset())
    QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  return QT_OK;
}

extern "C" qt_status qt_scba_solve(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                                   const qt_contacts* c, const double* V, double spindeg,
                                   double alpha, double tol, int max_iter, qt_precision prec,
                                   unsigned flags, double* sigma_r, double* sigma_lesser,
                                   double* sigma_greater, double* residuals, int* iters,
                                   double* currents) {
  Problem pb;
  GwGrid g;
  long long hn, h1n;
  QT_TRY(gw_setup(ctx, dev, E, nE, c, prec, flags, pb, g, hn, h1n));
  if (!V || !sigma_r || !sigma_lesser || !sigma_greater || max_iter <= 0)
    QT_FAIL(QT_ERR_ARG, "bad SCBA arguments");
  const long long npts = (long long)g.nk * nE;
  const long long cnt = npts * dev->nx * dev->nm * dev->nm;
  GwBuffers w{};
  GwAlloc hold;
  QT_TRY(gw_alloc(ctx, cnt, npts, g.nk, w, hold));
  cudaStream_t s = ctx->stream;
  double2* SR = reinterpret_cast<double2*>(sigma_r);
  double2* SL = reinterpret_cast<double2*>(sigma_lesser);
  double2* SG = reinterpret_cast<double2*>(sigma_greater);
  // terminal currents of each map's RGF, written as Id_iteration.dat does
  // (src/gw_mod.f90:413-428): sum_E tre and sum_E tr (the caller's tr/tre are the
  // routine's tre/tr, :376-380) x dE e0^2 spindeg / (2 pi hbar nk), with the
  // reference's constants (src/static.f90:10,14; src/fft_mod.f90:19)
  GwCurrents cur;
  std::vector<double> htr, htre;
  double dE = 0.0;
  if (currents) {
    cur.tre = w.sums + 8;
    cur.tr = cur.tre + npts;
    htr.resize(npts);
    htre.resize(npts);
    double e2[2] = {0, 0};
    cudaMemcpyAsync(e2, E, sizeof(e2), cudaMemcpyDeviceToHost, s);
    QT_CUDA_TRY(cudaStreamSynchronize(s));
    dE = e2[1] - e2[0];
  }
  const double e0 = 1.6022e-19, hbar = 1.0546e-34, tpi = 3.14159265359 * 2.0;
  const double ifac = dE * e0 / tpi / hbar * e0 * spindeg / g.nk;
  int it = 0;
  for (; it < max_iter; ++it) {
    QT_TRY(gw_map(ctx, pb, g, reinterpret_cast<const cd*>(V), spindeg, reinterpret_cast<cd*>(SR),
                  reinterpret_cast<cd*>(SL), w, hn, h1n, cur));
    if (currents) {
      cudaMemcpyAsync(htre.data(), cur.tre, npts * sizeof(double), cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(htr.data(), cur.tr, npts * sizeof(double), cudaMemcpyDeviceToHost, s);
      QT_CUDA_TRY(cudaStreamSynchronize(s));
      double a = 0.0, b = 0.0;
      for (long long e = 0; e < npts; ++e) { a += htre[e]; b += htr[e]; }
      currents[2 * it] = a * ifac;
      currents[2 * it + 1] = b * ifac;
    }
    cudaMemsetAsync(w.sums, 0, 2 * sizeof(double), s);
    qt::gw_residual(cnt, reinterpret_cast<double2*>(w.NL), SL, reinterpret_cast<double2*>(w.NG),
                    SG, w.sums, s);
    double h[2];
    cudaMemcpyAsync(h, w.sums, sizeof(h), cudaMemcpyDeviceToHost, s);
    QT_CUDA_TRY(cudaStreamSynchronize(s));
    const double r = std::sqrt(h[0]) / std::max(std::sqrt(h[1]), 1e-300);
    if (residuals) residuals[it] = r;
    // linear mixing (src/gw_mod.f90:747-749)
    qt::gw_mix(cnt, alpha, SR, reinterpret_cast<double2*>(w.NR), s);
    qt::gw_mix(cnt, alpha, SL, reinterpret_cast<double2*>(w.NL), s);
    qt::gw_mix(cnt, alpha, SG, reinterpret_cast<double2*>(w.NG), s);
    if (r <= tol) { ++it; break; }
  }
  if (iters) *iters = it;
  QT_CUDA_TRY(cudaStreamSynchronize(s));
  if (prec != QT_PREC_FP64 && qt::oz_timeouts_and_reset())
    QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  return QT_OK;
}

// e-photon self-energy in the monochromatic approximation
// (calc_sigma_ephoton_monochromatic_ext, src/gw_mod.f90:1075-1122): for every energy
// and slab, Sigma^{<,>} = scale M [G^{<,>}(E - hw) + G^{<,>}(E + hw)] M with M the slab's
// interaction block, Sigma^R = i Im(Sigma^> - Sigma^<)/2.  The shifted sum, scaled in FP64,
// is one elementwise pass (written into sigma_r, which is computed last), then two batched
// block products per component.
extern "C" qt_status qt_ephoton_sigma(qt_ctx* ctx, int nm, int nx, int nE, int nop, int halo,
                                      const double* M, const double* G_lesser,
                                      const double* G_greater, double scale, qt_precision prec,
                                      unsigned flags, double* sigma_r, double* sigma_lesser,
                                      double* sigma_greater) {
  if (!ctx || !M || !G_lesser || !G_greater || !sigma_r || !sigma_lesser || !sigma_greater ||
      nm <= 0 || nx <= 0 || nE <= 0 || nop < 0)
    QT_FAIL(QT_ERR_ARG, "bad e-photon arguments");
  if (!(flags & QT_FLAG_DEVICE_POINTERS)) QT_FAIL(QT_ERR_UNSUPPORTED, "device pointers required");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec != QT_PREC_FP64 && nm > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "split-precision path needs nm <= 384");
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const long long nm2 = (long long)nm * nm, nblk = (long long)nE * nx, cnt = nblk * nm2;
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes,
                (size_t)cnt * sizeof(cd) + (size_t)nblk * 256 * sizeof(int) + 4096));
  Arena ar{reinterpret_cast<char*>(ctx->arena), ctx->arena_bytes, 0};
  cd* one = ar.take<cd>(1);
  cd* T = ar.take<cd>((size_t)cnt);
  int* scales = ar.take<int>((size_t)nblk * 256);
  if (!one || !T || !scales) QT_FAIL(QT_ERR_NOMEM, "arena exhausted (e-photon)");
  const cd h1{1.0, 0.0};
  cudaMemcpyAsync(one, &h1, sizeof(cd), cudaMemcpyHostToDevice, s);
  Ops<double2> op{s, nm, prec};
  op.slices = 7;  // FP64-grade digits on the split path, as for the screened interaction
  op.one = one;
  op.scales = scales;
  op.P = nblk;
  op.prof = &ctx->prof;
  const BatchRef Mr = ref(M, nm2, nm, nx);  // block b = e*nx + x uses M[x]
  auto blk = [&](const void* p) { return ref(p, nm2, nm); };
  double2* A = reinterpret_cast<double2*>(sigma_r);
  const double* G[2] = {G_lesser, G_greater};
  double* out[2] = {sigma_lesser, sigma_greater};
  for (int c = 0; c < 2; ++c) {
    cudaError_t e = qt::photon_shift_sum((long long)nx * nm2, nE, nop, halo, scale,
                                         reinterpret_cast<const double2*>(G[c]), A, s);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    QT_TRY(op.gemm(Mr, qt::OP_N, blk(A), qt::OP_N, blk(T), nblk));
    QT_TRY(op.gemm(blk(T), qt::OP_N, Mr, qt::OP_N, blk(out[c]), nblk));
  }
  cudaError_t e = qt::photon_retarded(cnt, reinterpret_cast<const double2*>(sigma_lesser),
                                      reinterpret_cast<const double2*>(sigma_greater),
                                      reinterpret_cast<double2*>(sigma_r), s);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  if ((flags & QT_FLAG_SYNC) || prec != QT_PREC_FP64) QT_CUDA_TRY(cudaStreamSynchronize(s));
  if (prec != QT_PREC_FP64 && qt::oz_timeouts_and_reset())
    QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  return QT_OK;
}

extern "C" qt_status qt_corr_batch(qt_ctx* ctx, int n, int64_t nseries, const double* X,
                                   const double* Y, double* Z, int mode, unsigned flags) {
  if (!ctx || !X || !Y || !Z || n <= 0 || nseries <= 0 || (mode != 0 && mode != 1))
    QT_FAIL(QT_ERR_ARG, "bad correlation arguments");
  if (!(flags & QT_FLAG_DEVICE_POINTERS)) QT_FAIL(QT_ERR_UNSUPPORTED, "device pointers required");
  if (2 * n > 4096) QT_FAIL(QT_ERR_UNSUPPORTED, "n <= 2048");
  cudaSetDevice(ctx->device);
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, 2048 * sizeof(double2) + 256));
  double2* tw = reinterpret_cast<double2*>(ctx->arena);
  cudaError_t e = qt::gw_twiddles(tw, ctx->stream);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  qt::CorrConvArgs a{};
  a.n = n; a.nm = 1; a.nseries = nseries; a.estride = nseries;
  a.X = X; a.Y = Y; a.Z = Z; a.corr = mode == 0; a.scale_re = 1.0;
  e = qt::zcorrconv(a, tw, ctx->stream);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return QT_OK;
}

// ---- GW map stages on one rank's share (the energies <-> (i, j) exchange in between is
// the caller's: energies_to_ijs_2, src/gw_mod.f90:41-73, and its inverse)
namespace {

qt_status series_setup(qt_ctx* ctx, int n, int64_t nseries, unsigned flags,
                       qt::CorrConvArgs& c, double2*& tw) {
  if (n < 2 || nseries <= 0) QT_FAIL(QT_ERR_ARG, "need n >= 2 energies and nseries > 0");
  if (!(flags & QT_FLAG_DEVICE_POINTERS)) QT_FAIL(QT_ERR_UNSUPPORTED, "device pointers required");
  if (2 * n > 4096) QT_FAIL(QT_ERR_UNSUPPORTED, "n <= 2048 (FFT length 4096)");
  cudaSetDevice(ctx->device);
  QT_TRY(ensure(ctx->arena, ctx->arena_bytes, 2048 * sizeof(double2) + 256));
  tw = reinterpret_cast<double2*>(ctx->arena);
  cudaError_t e = qt::gw_twiddles(tw, ctx->stream);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  c = qt::CorrConvArgs{};
  c.n = n; c.nm = 1; c.nseries = nseries; c.estride = nseries;
  // the context's k-point grid: arrays [nk][n][nseries], the k-pair sums of the caller's
  // kmode; the band is applied on the blocks (qt_gw_screened, qt_gw_sigma_post)
  c.nky = ctx->gw_nky; c.nkz = ctx->gw_nkz; c.nk = c.nky * c.nkz;
  c.kstride = (long long)n * nseries;
  return QT_OK;
}

qt_status series_run(qt_ctx* ctx, const qt::CorrConvArgs& c, const double2* tw, const double* X,
                     const double* Y, double* Z, int corr, int conjY, int imX, int imY,
                     int acc, double sr, double si) {
  qt::CorrConvArgs a = c;
  a.kmode = corr ? 1 : 2;  // P sums over k at fixed q, Sigma over q at fixed k
  a.X = X; a.Y = Y; a.Z = Z; a.corr = corr; a.conjY = conjY;
  a.imagX = imX; a.imagY = imY; a.accumulate = acc; a.scale_re = sr; a.scale_im = si;
  cudaError_t e = qt::zcorrconv(a, tw, ctx->stream);
  if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
  return QT_OK;
}

}  // namespace

extern "C" qt_status qt_gw_polarization(qt_ctx* ctx, int n, int64_t nseries, const double* GR,
                                        const double* GL, const double* GG, const double* GLt,
                                        const double* GGt, double scale, double* PR,
                                        double* PL, double* PG, unsigned flags) {
  if (!ctx || !GR || !GL || !GG || !GLt || !GGt || !PR || !PL || !PG)
    QT_FAIL(QT_ERR_ARG, "null polarisation array");
  qt::CorrConvArgs c;
  double2* tw;
  QT_TRY(series_setup(ctx, n, nseries, flags, c, tw));
  // P = -i scale corr(...) of the Re-zeroed G (src/gw_mod.f90:444-446, 495-519)
  if (c.nk == 1) {  // packed transforms, as qt_gw_step
    qt::GwFusedArgs a{};
    a.n = n; a.nm = 1; a.nseries = nseries; a.estride = nseries;
    a.GR = GR; a.GL = GL; a.GG = GG; a.GLt = GLt; a.GGt = GGt;
    a.PR = PR; a.PL = PL; a.PG = PG;
    a.scale_re = 0.0; a.scale_im = -scale;
    cudaError_t e = qt::gw_polarization_packed(a, tw, ctx->stream);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return QT_OK;
  }
  QT_TRY(series_run(ctx, c, tw, GL, GGt, PL, 1, 0, 1, 1, 0, 0.0, -scale));
  QT_TRY(series_run(ctx, c, tw, GG, GLt, PG, 1, 0, 1, 1, 0, 0.0, -scale));
  // P^R = corr(G^<, conj G^R) + corr(G^R, G^<t), one inverse transform (as qt_gw_step)
  qt::CorrConvArgs a = c;
  a.X2 = GR; a.Y2 = GLt;
  QT_TRY(series_run(ctx, a, tw, GL, GR, PR, 1, 1, 1, 1, 0, 0.0, -scale));
  if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return QT_OK;
}

extern "C" qt_status qt_gw_screened(qt_ctx* ctx, int nm, int64_t nblocks, const double* V,
                                    const double* PR, const double* PL, const double* PG,
                                    double* WR, double* WL, double* WG, qt_precision prec,
                                    unsigned flags) {
  if (!ctx || !V || !PR || !PL || !PG || !WR || !WL || !WG || nm <= 0 || nblocks <= 0)
    QT_FAIL(QT_ERR_ARG, "bad screened-interaction arguments");
  if (!(flags & QT_FLAG_DEVICE_POINTERS)) QT_FAIL(QT_ERR_UNSUPPORTED, "device pointers required");
  if (!valid_prec(prec)) QT_FAIL(QT_ERR_ARG, "unknown precision");
  if (prec != QT_PREC_FP64 && nm > MAX_SPLIT)
    QT_FAIL(QT_ERR_UNSUPPORTED, "split-precision path needs nm <= 384");
  if (WR == PL || WR == PG || WL == PR || WL == PG || WG == PR || WG == PL)
    QT_FAIL(QT_ERR_ARG, "each W may alias only its own P (W^R -> P^R, W^< -> P^<, W^> -> P^>)");
  if (flags & QT_FLAG_V_PER_SLAB)
    QT_FAIL(QT_ERR_UNSUPPORTED, "per-slab Coulomb blocks: qt_gw_step / qt_scba_solve");
  const int nk = ctx->gw_nky * ctx->gw_nkz;
  if (nblocks % nk) QT_FAIL(QT_ERR_ARG, "nblocks must cover the nk k-points equally");
  cudaSetDevice(ctx->device);
  // FP64-grade digits on the split path, as inside qt_gw_step; group q of the blocks takes
  // V block q
  const long long nb = nblocks / nk, nm2 = (long long)nm * nm;
  auto P = [&](const double* a, int q) { return reinterpret_cast<const cd*>(a) + q * nb * nm2; };
  auto W = [&](double* a, int q) { return reinterpret_cast<cd*>(a) + q * nb * nm2; };
  for (int q = 0; q < nk; ++q)
    QT_TRY(gw_screened_blocks(ctx, nm, nb, prec, env_int("QT_LEAD_SLICES", 7),
                              reinterpret_cast<const cd*>(V) + q * nm2, P(PR, q), P(PL, q),
                              P(PG, q), W(WR, q), W(WL, q), W(WG, q), ctx->gw_ndiag));
  QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (prec != QT_PREC_FP64 && qt::oz_timeouts_and_reset())
    QT_FAIL(QT_ERR_CUDA, "tensor-core kernel wait timed out");
  return QT_OK;
}

extern "C" qt_status qt_gw_selfenergy(qt_ctx* ctx, int n, int64_t nseries, const double* GR,
                                      const double* GL, const double* GG, const double* WR,
                                      const double* WL, const double* WG, double scale,
                                      double* SR, double* SL, double* SG, unsigned flags) {
  if (!ctx || !GR || !GL || !GG || !WR || !WL || !WG || !SR || !SL || !SG)
    QT_FAIL(QT_ERR_ARG, "null self-energy array");
  qt::CorrConvArgs c;
  double2* tw;
  QT_TRY(series_setup(ctx, n, nseries, flags, c, tw));
  // Sigma = i scale conv(...) with the Re-zeroed G (src/gw_mod.f90:646-698)
  if (c.nk == 1) {  // packed transforms, as qt_gw_step
    qt::GwFusedArgs a{};
    a.n = n; a.nm = 1; a.nseries = nseries; a.estride = nseries;
    a.GR = GR; a.GL = GL; a.GG = GG; a.WR = WR; a.WL = WL; a.WG = WG;
    a.SR = SR; a.SL = SL; a.SG = SG;
    a.scale_re = 0.0; a.scale_im = scale;
    cudaError_t e = qt::gw_selfenergy_packed(a, tw, ctx->stream);
    if (e != cudaSuccess) QT_FAIL(QT_ERR_CUDA, cudaGetErrorString(e));
    if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return QT_OK;
  }
  QT_TRY(series_run(ctx, c, tw, GL, WL, SL, 0, 0, 1, 0, 0, 0.0, scale));
  QT_TRY(series_run(ctx, c, tw, GG, WG, SG, 0, 0, 1, 0, 0, 0.0, scale));
  // Sigma^R = conv(G^<, W^R) + conv(G^R, W^< + W^R), one inverse transform (as qt_gw_step)
  qt::CorrConvArgs a = c;
  a.X2 = GR; a.Y2 = WL; a.Y2b = WR;
  QT_TRY(series_run(ctx, a, tw, GL, WR, SR, 0, 0, 1, 0, 0, 0.0, scale));
  if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return QT_OK;
}

extern "C" qt_status qt_gw_sigma_post(qt_ctx* ctx, int nm, int nx, int nE, double* SR,
                                      double* SL, double* SG, unsigned flags) {
  if (!ctx || !SR || !SL || !SG || nm <= 0 || nx <= 0 || nE <= 0)
    QT_FAIL(QT_ERR_ARG, "bad self-energy post-processing arguments");
  if (!(flags & QT_FLAG_DEVICE_POINTERS)) QT_FAIL(QT_ERR_UNSUPPORTED, "device pointers required");
  cudaSetDevice(ctx->device);
  const long long nk = (long long)ctx->gw_nky * ctx->gw_nkz;
  QT_TRY(gw_post(ctx, nm, nx, nk * nE, reinterpret_cast<cd*>(SR), reinterpret_cast<cd*>(SL),
                 reinterpret_cast<cd*>(SG), ctx->gw_ndiag));
  if (flags & QT_FLAG_SYNC) QT_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return QT_OK;
}
