// Internal launch interfaces of the batched kernels (not part of the C-ABI).
#pragma once
#include "qt_common.cuh"

namespace qt {

enum { OP_N = 0, OP_C = 1, OP_T = 2 };

// every kernel launch of the library is counted (reported by qt_kernel_launches)
void count_launch(long long n = 1);

// C_b = alpha * op(A_b) op(B_b) + beta * D_b + z_b * I   (m x n result, inner k)
struct GemmArgs {
  int m, n, k;
  BatchRef A, B, C, D, Z;  // D.p / Z.p may be null; Z entries are single complex
  int opA, opB;
  double alpha_re, alpha_im, beta_re, beta_im;
  long long batch;
  const unsigned char* active;  // optional per-batch mask: skip entry when 0
  int* scales;  // split-precision scratch: batch x 256 ints (row / column exponents)
  // split-precision waits that time out are counted here; null: the library-wide counter
  // read by oz_timeouts_and_reset()
  int* timeouts = nullptr;
};

cudaError_t zgemm_f64(const GemmArgs& a, cudaStream_t s);

// Split-precision (Ozaki-style bf16 digits) tensor-core GEMM; same contract.
//   slices: digits per operand row/column (8 bits each)
//   levels: highest digit-product level kept (level = i + j)
cudaError_t zgemm_oz(const GemmArgs& a, int slices, int levels, cudaStream_t s);
// complex64 in/out variant (3 or 4 digits): the split-precision RGF sweep
cudaError_t zgemm_oz_c64(const GemmArgs& a, int slices, cudaStream_t s);
// number of bounded waits that timed out in the tensor-core kernel since the last call
int oz_timeouts_and_reset();

// X_b = inv(A_b), Gauss-Jordan with partial pivoting; status_b |= PT_SINGULAR
// on a zero or non-finite pivot.  X may alias A.
struct InvArgs {
  int n;
  BatchRef A, X;
  long long batch;
  int* status;                  // per batch (may be null)
  const unsigned char* active;  // optional mask
};
cudaError_t zinv_f64(const InvArgs& a, cudaStream_t s);
// the same FP64 elimination for storage TC; complex64 blocks go through the complex128
// workspace W (entry b at W + b * wst)
template <typename TC>
cudaError_t zinv_f64_ws(const InvArgs& a, cd* W, long long wst, cudaStream_t s);
// flag[b] = active[b] && (||R_b||_F > tol or non-finite), R_b n x n; *count += flags
template <typename TC>
cudaError_t zinv_guard(int n, long long batch, BatchRef R, const unsigned char* active,
                       double tol, unsigned char* flag, int* count, cudaStream_t s);
// FP32 elimination in shared memory (n <= 128); TC = storage of A and X
template <typename TC>
cudaError_t zinv_f32(const InvArgs& a, cudaStream_t s);

// ---- elementwise helpers, TC = double2 (complex128) or float2 (complex64);
// n x n column-major blocks; diagonal shifts Z are always complex128 scalars.
// Y_b = alpha*X_b + beta*W_b + z_b*I   (X or W may be null -> 0)
template <typename TC>
cudaError_t zaxpby(int n, long long batch, BatchRef X, double alpha_re, double alpha_im,
                   BatchRef W, double beta_re, double beta_im, BatchRef Z, BatchRef Y,
                   const unsigned char* active, cudaStream_t s);
// Y_b = c * (X_b - X_b^+) + W_b  (W may be null)
template <typename TC>
cudaError_t zantiherm(int n, long long batch, BatchRef X, double c_re, double c_im, BatchRef W,
                      BatchRef Y, cudaStream_t s);
// Y_b = X_b^+
template <typename TC>
cudaError_t zdagger(int n, long long batch, BatchRef X, BatchRef Y, cudaStream_t s);
// Y1_b += X_b; Y2_b += X_b  (Y1, Y2 and X distinct)
template <typename TC>
cudaError_t zadd2(int n, long long batch, BatchRef X, BatchRef Y1, BatchRef Y2,
                  const unsigned char* active, cudaStream_t s);
// out_b = sum_ij |X_b(i,j)|  (the reference's Sancho error measure), exact to FP64 where it
// decides the comparison with `near` (the decimation's tolerance), a few 1e-7 elsewhere
template <typename TC>
cudaError_t zabssum(int n, long long batch, BatchRef X, double* out, const unsigned char* active,
                    double near, cudaStream_t s);
// out_b = sign * Re(f Tr[K Y1] - (f-1) Tr[K Y2]), K = -(X - X^+), f = fermi[b]
template <typename TC>
cudaError_t ztrace_current(int n, long long batch, BatchRef X, BatchRef Y1, BatchRef Y2,
                           double sign, const double* fermi, double* out, cudaStream_t s);
// out_b = scale * Re Tr[X_b Y_b]
template <typename TC>
cudaError_t ztrace_prod(int n, long long batch, BatchRef X, BatchRef Y, double scale, double* out,
                        cudaStream_t s);
// Bond current between slabs l and l+1 from T1 = g H^+ G^<_{l+1} (nl x nq), the
// coupling H = H_{l+1,l} (nq x nl) and A = G_{l+1} H g^< (nq x nl):
// out[b*ostride + ooff] = scale * 2 (-Re Tr[T1 H] + Re Tr[H^+ A]); T1 may be null
template <typename TC>
cudaError_t zbond_trace(int nl, int nq, long long batch, BatchRef T1, BatchRef H, BatchRef A,
                        double scale, double* out, long long ostride, long long ooff,
                        cudaStream_t s);
// Y_b = f[b] * X_b + W_b   (W may be null)
template <typename TC>
cudaError_t zscale_add(int n, long long batch, BatchRef X, const double* f, BatchRef W, BatchRef Y,
                       cudaStream_t s);
// out[b*ostride + ooff + i] = X_b(i,i)   (complex128 output)
template <typename TC>
cudaError_t zdiag(int n, long long batch, BatchRef X, double* out, long long ostride,
                  long long ooff, cudaStream_t s);
// out[b*ostride + ooff + i] = Y_b(i,i) + X_b(i,i) - conj(X_b(i,i))   (diag of G^< + G - G^+)
template <typename TC>
cudaError_t zdiag_greater(int n, long long batch, BatchRef X, BatchRef Y, double* out,
                          long long ostride, long long ooff, cudaStream_t s);
template <typename TC>
cudaError_t zcopy(int n, long long batch, BatchRef X, BatchRef Y, cudaStream_t s);
// storage conversion complex128 <-> complex64
template <typename TS, typename TD>
cudaError_t zconvert(int n, long long batch, BatchRef X, BatchRef Y, cudaStream_t s);
// status_b |= PT_NONFINITE if any element of X_b is not finite
template <typename TC>
cudaError_t zcheck_finite(int n, long long batch, BatchRef X, int* status, cudaStream_t s);

// ---- GW/SCBA (gw.cu): energy series of element (i,j) of slab ix, arrays [nE][nx][nm*nm]
struct CorrConvArgs {
  int n;              // energies per series
  int nm;             // block size
  long long nseries;  // series per k-point (nx * nm * nm)
  long long estride;  // element stride between consecutive energies (nx * nm * nm)
  const void* X;
  const void* Y;
  void* Z;
  int corr;           // 1: correlation (Y reversed), 0: convolution
  int transY;         // Y series is the transposed element (j, i)
  int conjY, imagX, imagY;  // conj(Y); Re(X) := 0; Re(Y) := 0 (applied before conj)
  int accumulate;     // Z += result
  double scale_re, scale_im;
  // optional second term, summed before the inverse transform:
  //   Z = scale (op(X, Y) + op(X2, Y2 + Y2b))   (X2 null: one term; Y2b may be null)
  // with its own transposition / conjugation of Y2 (imagX / imagY apply to both terms).
  // With one k-point (or kmode 0), Z may alias X or X2: a series is read completely
  // before it is written.
  const void* X2 = nullptr;
  const void* Y2 = nullptr;
  const void* Y2b = nullptr;
  int transY2 = 0, conjY2 = 0;
  // k-points (src/gw_mod.f90:476-512, 653-690): the arrays hold nk = nky * nkz blocks of
  // nseries series, kstride elements apart, and the output covers all nk * nseries.
  //   kmode 0: output k from X, Y at k;
  //   kmode 1: output q = sum over k of op(X_k, Y_kd(k,q))   (polarisation);
  //   kmode 2: output k = sum over q of op(X_kd(k,q), Y_q)   (self-energy).
  // With nk > 1 and kmode != 0, Z must not alias any input.
  int nk = 1, nky = 1, nkz = 1, kmode = 0;
  long long kstride = 0;
  // band (:471-475): series whose element (i, j) has |i - j| > ndiag are written as zero
  // (ndiag < 0: none).  A series' element is ij0 + (series mod nel) in column-major order
  // (nel = 0: nm * nm, the full blocks of qt_gw_step).
  int ndiag = -1;
  long long nel = 0, ij0 = 0;
  int L, logL;        // set by the launcher
};
// P and Sigma of one k-point with packed transforms, one energy series (matrix element) per
// CTA: every input of P and every G of Sigma is purely imaginary once Re G is zeroed, so two
// such series share one complex FFT (z = a + i b of the real sequences a, b; their transforms
// follow from Z(k) and conj Z(L - k)).  P takes 6 FFTs per element for the 11 of three
// separate correlations, Sigma 8 for 11.  Layout and band as CorrConvArgs (nk = 1).
struct GwFusedArgs {
  int n, nm;
  long long nseries, estride;
  long long nel = 0, ij0 = 0;
  int ndiag = -1;
  // polarisation: P^< = s corr(G^<, G^>t), P^> = s corr(G^>, G^<t),
  // P^R = s [corr(G^<, conj G^R) + corr(G^R, G^<t)]; with GLt / GGt null the transposed
  // partner is element (j, i) of G^< / G^> (full blocks)
  const void *GR = nullptr, *GL = nullptr, *GG = nullptr, *GLt = nullptr, *GGt = nullptr;
  void *PR = nullptr, *PL = nullptr, *PG = nullptr;
  // self-energy: S^< = s conv(G^<, W^<), S^> = s conv(G^>, W^>),
  // S^R = s [conv(G^<, W^R) + conv(G^R, W^< + W^R)]; S may overwrite G (each CTA reads its
  // series completely before writing them)
  const void *WR = nullptr, *WL = nullptr, *WG = nullptr;
  void *SR = nullptr, *SL = nullptr, *SG = nullptr;
  double scale_re = 0.0, scale_im = 0.0;
  int L = 0, logL = 0;  // set by the launcher
};
cudaError_t gw_polarization_packed(GwFusedArgs a, const double2* tw, cudaStream_t s);
cudaError_t gw_selfenergy_packed(GwFusedArgs a, const double2* tw, cudaStream_t s);
cudaError_t gw_twiddles(double2* tw, cudaStream_t s);  // 2048 entries exp(-2 pi i k / 4096)
cudaError_t zcorrconv(CorrConvArgs a, const double2* tw, cudaStream_t s);
cudaError_t gw_sigma_post(int nm, long long nblocks, double2* SR, double2* SL, double2* SG,
                          cudaStream_t s);
cudaError_t gw_residual(long long count, const double2* nl, const double2* ol, const double2* ng,
                        const double2* og, double* sums, cudaStream_t s);
cudaError_t gw_mix(long long count, double alpha, double2* S, const double2* N, cudaStream_t s);
// zero the elements |i - j| > ndiag of nblocks column-major nm x nm blocks, bstride
// elements apart (0: nm * nm), when ndiag >= 0
cudaError_t gw_band_zero(int nm, long long nblocks, int ndiag, double2* A, cudaStream_t s,
                         long long bstride = 0);
// e-photon self-energy pieces (src/gw_mod.f90:1075-1122): A[e] = scale (G[e-nop] + G[e+nop])
// per block of per = nx*nm*nm elements (halo != 0: G carries nop extra energies on each
// side), and Sigma^R = i Im(Sigma^> - Sigma^<)/2
cudaError_t photon_shift_sum(long long per, long long nE, int nop, int halo, double scale,
                             const double2* G, double2* A, cudaStream_t s);
cudaError_t photon_retarded(long long count, const double2* SL, const double2* SG, double2* SR,
                            cudaStream_t s);

}  // namespace qt
