/*
 * qt_rgf.h -- C-ABI of the GB300 (sm_103a) batched recursive Green's function
 * library (libqtgpu.so).  Plain pointers and sizes only.
 *
 * Storage: every n x n block is complex128 COLUMN-MAJOR with interleaved
 * (re, im) doubles -- the memory image of Fortran complex(8) arrays, so a
 * Fortran caller passes its arrays unchanged through iso_c_binding.
 * Points are ordered energy-major, k-minor: p = ie*nk + ik, the loop order of
 * negf_solve (src/negf_mod.f90:115-116).
 *
 * Pointers are HOST pointers unless QT_FLAG_DEVICE_POINTERS is set, in which
 * case every array argument must be device memory of the context's GPU.
 */
#ifndef QT_RGF_H
#define QT_RGF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  QT_OK = 0,
  QT_ERR_ARG = 1,         /* invalid argument (sizes, null pointers)             */
  QT_ERR_CUDA = 2,        /* CUDA runtime error; see qt_last_error()             */
  QT_ERR_NOMEM = 3,       /* device allocation failed                           */
  QT_ERR_UNSUPPORTED = 4, /* configuration not supported (e.g. nm > 384 mixed)   */
  QT_ERR_POINTS = 5       /* finished, but at least one point has status != 0   */
} qt_status;

/* per-point status bits (qt_outputs.status) */
#define QT_PT_OK 0
#define QT_PT_SINGULAR 1              /* zero/non-finite pivot in a block inverse */
#define QT_PT_SANCHO_NOT_CONVERGED 2  /* decimation hit max_iter above tol        */
#define QT_PT_NONFINITE 4             /* NaN/Inf in an output block               */

typedef enum {
  QT_PREC_FP64 = 0,  /* complex128 on the FP64 pipes (plain path)                 */
  QT_PREC_MIXED = 1, /* Ozaki-split bf16 tensor-core GEMMs (tcgen05, FP32 TMEM
                        accumulation, exact leading digit levels), FP32 block LU +
                        one residual refinement; Sancho at FP64-grade digits.
                        The sweep stores complex64 blocks: H is resolved to
                        2^-24 relative, which near band edges (η -> 0) moves
                        spectra by up to ~1e-4 of their maximum               */
  QT_PREC_MIXED_FP64 = 2 /* the same tensor-core products with complex128
                        storage everywhere: 6-digit products (2^-44 relative)
                        in the sweep, 7 in the leads, FP32 block LU + three
                        refinements.  FP64-grade results at tensor-core rate  */
} qt_precision;
/* Both split precisions take blocks up to 384 orbitals (above 128 the products are
 * tiled and the inverses use the 2 x 2 block form).  A block whose FP32 elimination
 * leaves a first residual too large for the refinement to converge is eliminated
 * again in FP64 (see qt_ctx_inverse_fallbacks).                                 */

#define QT_FLAG_DEVICE_POINTERS 1u /* all arrays are device pointers            */
#define QT_FLAG_CAROLI 2u          /* also compute Caroli T(E) (qt_outputs.T)    */
#define QT_FLAG_SYNC 4u            /* synchronise the stream before returning   */
#define QT_FLAG_COMPLEX64 16u      /* qt_zgemm_batch: A, B, D, C are complex64
                                      (interleaved float pairs) device blocks;
                                      QT_PREC_MIXED, 4 digits, real alpha/beta */
#define QT_FLAG_SANCHO_RESET 8u    /* qt_sancho_batch: green_RGF_RS's decimation
                                      (src/gw_mod.f90:1440-1445): an entry not
                                      converged after max_iter steps restarts
                                      from H_SS = H_BB = H00                   */
#define QT_FLAG_V_PER_SLAB 32u     /* qt_gw_step, qt_scba_solve: V holds one
                                      Coulomb block per q and slab,
                                      [nk][nx][nm*nm], as the reference's
                                      Vii(nm, nm, nx, nk) (src/gw_mod.f90:84) */

/* Reference-quirk switches (default 0 = the behaviour that produced the
 * reference's test_cnt/ outputs).                                            */
#define QT_QUIRK_CPU_FERMI 1u    /* contact Fermi/temperature pairing, tr sign
                                    and bond-current form of
                                    rgf_variableblock_forward (src/rgf_mod.f90:
                                    100,182,196-202,215-221,258)             */
#define QT_QUIRK_GLP_ZERO 2u     /* G^> recursion seeded with Glp == 0 as in
                                    src/cuda_rgf_mod.f90:78,351-372          */
#define QT_QUIRK_BACK_H1I_NEXT 4u /* backward step couples l,l+1 through
                                    H1i(l+1) instead of the reference's H1i(l)
                                    (identical for slab-independent coupling) */
#define QT_QUIRK_GW_SANCHO_RESET 8u /* lead decimation of green_RGF_RS
                                    (src/gw_mod.f90:1440-1445): a point whose
                                    decimation is not converged after
                                    sancho_max_iter steps takes H_SS = H_BB =
                                    H00, i.e. the isolated-slab surface
                                    function; off by default (the points keep
                                    their last iterate and are flagged)     */

typedef struct qt_ctx qt_ctx;

/* Replaces cuda_rgf_init(nm) / cuda_rgf_finish() (src/cuda_rgf_mod.f90:32-51):
 * the context owns a CUDA stream and grow-only device scratch; contexts are
 * independent (no module-level state, unlike src/cuda_rgf_mod.f90:24-28).  */
qt_status qt_ctx_create(qt_ctx** ctx, int device);
qt_status qt_ctx_destroy(qt_ctx* ctx);
qt_status qt_ctx_sync(qt_ctx* ctx);
/* Launch on `stream` (a cudaStream_t, e.g. the caller framework's current
 * stream, 0 = the legacy default stream) instead of the context's own stream,
 * so that the caller's work on its buffers is ordered with the library's;
 * use_own != 0 returns to the context's own stream.  Synchronises the stream
 * in use before switching.  Networks (qt_mlp) launch on their context's
 * current stream and must be destroyed before their context.               */
qt_status qt_ctx_set_stream(qt_ctx* ctx, void* stream, int use_own);
/* Bound (bytes) on the per-wave device scratch; default 48 GiB.            */
qt_status qt_ctx_set_scratch_limit(qt_ctx* ctx, int64_t bytes);
/* Batch schedule: (E, k) points solved together in one wave of the sweeps
 * (qt_rgf_solve, qt_rgf_solve_vb, qt_gw_step, qt_scba_solve), rounded down to
 * whole energies (multiples of nk) and bounded by the scratch limit; 0 (the
 * default) = 608, four work items per SM of a 152-SM GPU.  Results do not
 * depend on it.  quantum_transport_gb300/autotune.py picks it by measurement. */
qt_status qt_ctx_set_wave_points(qt_ctx* ctx, int64_t points);
/* Message of the last error on this thread ("" if none).                   */
const char* qt_last_error(void);
/* Library version string.                                                   */
const char* qt_version(void);

/* Instrumentation (no counterpart in the reference, which only prints
 * omp_get_wtime phase times, src/cuda_rgf_mod.f90:87-412).
 * qt_kernel_launches: kernels launched by this library since load.
 * qt_ctx_profile(enable): record CUDA events around every block product and
 *   inverse on the context's stream, and around the phases of each GW map.
 * qt_ctx_profile_read(kind): launches, summed device time (ms) and the
 *   algorithmic / executed-tensor flops of one kind since the last read:
 *   0 complex64 split product, 1 complex128 split product, 2 FP64 product,
 *   3 FP32 inverse, 4 FP64 inverse; GW map phases (qt_gw_step, qt_scba_solve;
 *   flops 0, products and inverses inside them also counted above): 5 the RGF
 *   of G, 6 the energy correlations / convolutions of P and Sigma, 7 the
 *   screened interaction W, 8 Sigma's band, recombination and symmetrisation.
 * qt_ctx_stream: the context's cudaStream_t (as void*).                    */
int64_t qt_kernel_launches(void);
qt_status qt_ctx_profile(qt_ctx* ctx, int enable);
qt_status qt_ctx_profile_read(qt_ctx* ctx, int kind, int64_t* launches, double* ms,
                              double* alg_flops, double* tensor_flops);

/* Instrumentation: how many block inverses the split path redid in FP64.  Each
 * split-path inverse starts from an FP32 elimination and refines it; when the first
 * residual I - A X is too large for the refinement to reach storage precision (an
 * ill-conditioned block), the entry is eliminated again in FP64.  reset != 0 zeroes
 * the counter after reading.                                                  */
qt_status qt_ctx_inverse_fallbacks(qt_ctx* ctx, int64_t* count, int reset);
qt_status qt_ctx_stream(qt_ctx* ctx, void** stream);

/* Block-tridiagonal device of nx slabs of constant block size nm at nk
 * transverse k-points (cuda_rgf_constblocksize's Hii(nx), H1i(nx+1), Sii(nx),
 * src/cuda_rgf_mod.f90:55; built per k by devH_build_fromWannierFile,
 * src/deviceHam_mod.f90:269-287).
 *   Hii block (k, l) at Hii + 2*(k*hii_kstride + l*hii_lstride) doubles
 *   H1i block (k, l) at H1i + 2*(k*h1i_kstride + l*h1i_lstride), l = 0..nx,
 *       H1i[l] = H_{l,l-1}; H1i[0] couples the left lead, H1i[nx] the right
 *   Sii: NULL => identity (the only case any reference driver uses)
 * A stride of 0 means "identical for all k" / "identical for all slabs".   */
typedef struct {
  int nm, nx, nk;
  const double* Hii;
  int64_t hii_kstride, hii_lstride;
  const double* H1i;
  int64_t h1i_kstride, h1i_lstride;
  const double* Sii;
  int64_t sii_kstride, sii_lstride;
} qt_device;

/* Contacts and Sancho-Rubio settings.  Reference values: eta_lead = 1e-5
 * (src/cuda_rgf_mod.f90:671), eta_interior = 0 (:68), sancho_max_iter = 50
 * (:670), sancho_tol = 1e-100 (:661), mu/temp from negf_solve (:82-85).      */
typedef struct {
  double mul, mur;       /* chemical potentials (eV)          */
  double templ, tempr;   /* temperatures (K)                  */
  double eta_lead;       /* Sancho Im(z)                      */
  double eta_interior;   /* Im(z) of interior slabs           */
  double sancho_tol;     /* exit when sum_ij |H_01(i,j)| < tol */
  int sancho_max_iter;
  unsigned quirks;       /* QT_QUIRK_* bits                   */
} qt_contacts;

/* Outputs, per point p (any pointer may be NULL = not wanted).
 *   tr, tre   [npts]  terminal-current spectra of cuda_rgf_constblocksize
 *                     (src/cuda_rgf_mod.f90:271-277, 403-407)
 *   T         [npts]  Caroli transmission (needs QT_FLAG_CAROLI)
 *   diag_gr/gl/gg [npts][nx*nm] complex128 diagonals of G^R, G^<, G^>
 *                     (the per-orbital data behind ldos/ndos/pdos,
 *                     src/negf_mod.f90:141-149)
 *   G_r, G_lesser, G_greater [npts][nx][nm*nm] full diagonal blocks
 *                     (cuda_rgf_constblocksize's G_r, G_lesser, G_greater)
 *   status    [npts]  QT_PT_* bits
 *   sancho_iters [npts][2] iterations of the left/right decimation
 *   bond_cur  [npts][nx-1] bond currents J_l = Re Tr Jdens_l between slabs l
 *                     and l+1 (0-based), Jdens_l = H^+ G^<_{l+1,l} - H G^<_{l,l+1}
 *                     with H = H_{l+1,l} (src/cuda_rgf_mod.f90:293-318); with
 *                     QT_QUIRK_CPU_FERMI the CPU routine's
 *                     Jdens_l = -2 H^+ G^<_{l+1,l} (src/rgf_mod.f90:215-221)
 *   Jdens     [npts][nx][nm*nm] the full Jdens_l blocks of
 *                     cuda_rgf_constblocksize; block nx-1 is zero as there
 *                     (qt_rgf_solve without QT_QUIRK_CPU_FERMI only)        */
typedef struct {
  double* tr;
  double* tre;
  double* T;
  double* diag_gr;
  double* diag_gl;
  double* diag_gg;
  double* G_r;
  double* G_lesser;
  double* G_greater;
  int* status;
  int* sancho_iters;
  double* bond_cur;
  double* Jdens;
} qt_outputs;

/* Batched ballistic/phonon RGF over nE energies x nk k-points: the whole
 * ``do ie / do ik / call cuda_rgf_constblocksize`` loop of negf_solve
 * (src/negf_mod.f90:115-127) in one call.
 *   E [nE] energies (eV)
 *   sigma_r_ph, sigma_lesser_ph: NULL (=> 0, the negf_solve case) or
 *       [npts][nx][nm*nm] complex128 scattering self-energies
 *       (cuda_rgf_constblocksize's sigma_r_ph / sigma_lesser_ph)         */
qt_status qt_rgf_solve(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                       const qt_contacts* contacts, const double* sigma_r_ph,
                       const double* sigma_lesser_ph, qt_precision prec, unsigned flags,
                       qt_outputs* out);

/* Slabs with different orbital counts: rgf_variableblock_forward
 * (src/rgf_mod.f90:46-269) over all nE x nk points.  Block l (0-based) has
 * nm[l] orbitals.
 *   Hii + hii_off[l]  H_ll, nm[l] x nm[l], column-major (+ ik * hii_kstride per k)
 *   H1i + h1i_off[l]  H1i[l] = H_{l,l-1}, nm[l] x nm[l-1], for 1 <= l < nx;
 *                     H1i[0], H1i[nx]: the left / right lead's own coupling
 *                     (nm[0] x nm[0], nm[nx-1] x nm[nx-1]) (+ ik * h1i_kstride)
 * Offsets in complex elements; nm, hii_off, h1i_off are host arrays.  The
 * backward step couples slabs l and l+1 through H_{l+1,l}: the reference's
 * H1i(l) (src/rgf_mod.f90:215-245) only fits equal neighbouring blocks.  The
 * right lead is decimated with H1i[nx] as in src/rgf_mod.f90:153.
 * Outputs: tr, tre, T [npts]; diag_gr / diag_gl / diag_gg packed
 * [npts][sum nm[l]] complex128; full blocks are not returned (must be NULL).
 * The split precisions need nm[l] <= 384 (blocks above 128 are tiled).     */
typedef struct {
  int nx, nk;
  const int* nm;
  const double* Hii;
  const int64_t* hii_off;
  int64_t hii_kstride;
  const double* H1i;
  const int64_t* h1i_off;
  int64_t h1i_kstride;
} qt_device_vb;

qt_status qt_rgf_solve_vb(qt_ctx* ctx, const qt_device_vb* dev, const double* E, int nE,
                          const qt_contacts* contacts, qt_precision prec, unsigned flags,
                          qt_outputs* out);

/* Slab blocks of a Wannier90 tight-binding model: w90_MAT_DEF
 * (src/wannierHam3d.f90:273-301) at nk transverse k-points in one launch.
 *   Hr     the model's H(R), Fortran Hr(nb, nb, nxr, nyr, nzr) complex128, with
 *          R ranges range = {xmin, xmax, ymin, ymax, zmin, zmax}
 *   cell   the cell vectors alpha, beta, gamm (3 x 3 doubles, Angstrom)
 *   kvec   [nk][3] Cartesian k vectors kx xhat + ky yhat + kz zhat (1/Angstrom)
 *   H00    [nk][nm*nm] H_ii of a slab of ns cells (nm = nb*ns), column-major
 *   H10    [nk][nm*nm] H_{i+1,i}
 * Host pointers unless QT_FLAG_DEVICE_POINTERS.  The outputs feed qt_rgf_solve
 * with hii_kstride = nm*nm.                                                */
qt_status qt_w90_blocks(qt_ctx* ctx, int nb, int ns, const int* range, const double* Hr,
                        const double* cell, int nk, const double* kvec, double* H00,
                        double* H10, unsigned flags);

/* Device blocks from a COO Hamiltonian: the blocksize branch of
 * devH_build_fromCOOfile (src/deviceHam_mod.f90:168-224), fed by the entries
 * load_COOmatrix reads (src/deviceHam_mod.f90:40-91).
 *   row, col    nnz indices, index_base 0 or 1
 *   h           nnz complex128 values; s the overlap values on the same
 *               entries, or NULL (then Sii = I)
 *   Hii, Sii    [nx][bs*bs] column-major; H1i [nx+1][bs*bs]
 * An entry of slab ix (row div bs) whose column lies in slab ix writes
 * Hii[mm,nn] = h and Hii[nn,mm] = conj(h); in slab ix+1 it writes
 * H1i(ix)[mm, nn-bs]; anything else is dropped.  H1i(nx) repeats H1i(nx-1).
 * Later entries win, as in the reference's serial loop; the result is
 * bit-exact and independent of thread order.  Host pointers unless
 * QT_FLAG_DEVICE_POINTERS.                                                 */
qt_status qt_coo_blocks(qt_ctx* ctx, int nx, int bs, long long nnz, const int* row,
                        const int* col, int index_base, const double* h, const double* s,
                        double* Hii, double* H1i, double* Sii, unsigned flags);

/* Single-point drop-in with the argument list of cuda_rgf_constblocksize
 * (src/cuda_rgf_mod.f90:53-59): contiguous (nm, nm, nx) arrays for Hii, Sii,
 * sigma_lesser_ph, sigma_r_ph, G_r, G_lesser, G_greater, Jdens and
 * (nm, nm, nx+1) for H1i; mu/T scalars (the reference broadcasts them into
 * constant nm x nm matrices, src/negf_mod.f90:78-85).  Host pointers; Sii,
 * the sigmas and Jdens may be NULL.  Runs in FP64.                         */
qt_status qt_rgf_constblocksize(qt_ctx* ctx, int nm, int nx, double En, double mul, double mur,
                                double templ, double tempr, const double* Hii, const double* H1i,
                                const double* Sii, const double* sigma_lesser_ph,
                                const double* sigma_r_ph, double* G_r, double* G_lesser,
                                double* G_greater, double* Jdens, double* tr, double* tre);

/* Batched Sancho-Rubio decimation, ``sancho(nm, E, S00, H00, H10, G00, GBB)``
 * (src/rgf_mod.f90:482; GPU variant src/cuda_rgf_mod.f90:657-765) for npts
 * independent leads.  H00/H10/S00 block b at ptr + 2*b*stride doubles (stride
 * 0 = shared); S00 NULL => identity.  G00/GBB [npts][nm*nm]; iters [npts].   */
qt_status qt_sancho_batch(qt_ctx* ctx, int nm, int npts, const double* E, const double* H00,
                          int64_t h00_stride, const double* H10, int64_t h10_stride,
                          const double* S00, int64_t s00_stride, double eta, double tol,
                          int max_iter, qt_precision prec, unsigned flags, double* G00,
                          double* GBB, int* iters, int* status);

/* Batched block product C_b = alpha op(A_b) op(B_b) + beta D_b (the
 * reference's MUL_C / zgemm, src/matrix_c.f90:615-660), square n x n blocks,
 * op 'N' / 'C' / 'T'.  Strides in complex elements (0 = shared block).  D may
 * be NULL.  prec selects the FP64 pipes or the tensor-core split product
 * with `slices` 8-bit digits per operand (ignored for FP64; 0 = default 4).
 * With QT_FLAG_COMPLEX64 the blocks are complex64 (the split sweep's storage)
 * and the pointers are read as float pairs.                                 */
qt_status qt_zgemm_batch(qt_ctx* ctx, int n, int batch, char opA, const double* A,
                         int64_t a_stride, char opB, const double* B, int64_t b_stride,
                         const double* alpha, const double* beta, const double* D,
                         int64_t d_stride, double* C, int64_t c_stride, qt_precision prec,
                         int slices, unsigned flags);

/* Batched block inverse (the reference's ``invert``, src/linalg.f90:42-62,
 * src/cuda_rgf_mod.f90:624-654).  X may equal A.  status [batch] gets
 * QT_PT_SINGULAR bits.  MIXED: FP32 elimination + one refinement step.   */
qt_status qt_zinv_batch(qt_ctx* ctx, int n, int batch, const double* A, int64_t a_stride,
                        double* X, int64_t x_stride, qt_precision prec, unsigned flags,
                        int* status);

/* Allocation-free split-precision block product.  No counterpart in the
 * reference: it exists for callers that must not allocate device memory --
 * hosts whose device memory belongs to another allocator (a framework's caching
 * pool, a Fortran code's OpenMP `target enter data` buffers) and latency-
 * critical loops where cudaMalloc/cudaFree would implicitly synchronise the
 * device.  Same product as qt_zgemm_batch with QT_PREC_MIXED (device pointers,
 * op 'N'/'C', real alpha/beta, n <= 128, slices 0 (=4), 4, 6 or 7), but its
 * scratch (256 scale exponents per batch entry) lives in a file-scope device
 * array of QT_NOALLOC_MAX_BATCH x 256 ints (512 KiB per GPU, held until the
 * process exits), and it needs no context: work goes on `stream`.
 *   - batch > QT_NOALLOC_MAX_BATCH is rejected with QT_ERR_ARG;
 *   - every call looks up the array's device address with
 *     cudaGetSymbolAddress (the caller's device current).  Under CUDA's
 *     default lazy module loading the first call on a device loads the
 *     library's device module, which can allocate module memory and
 *     synchronise: make one warm-up call outside latency-critical code and
 *     before any stream capture, or set CUDA_MODULE_LOADING=EAGER;
 *   - all calls share the array, so calls overlapping on the GPU race;
 *   - it calls no cudaMalloc, cudaFree or other allocating routine;
 *   - QT_OK means the work was enqueued.  A bounded wait inside the
 *     tensor-core kernel that runs out (4 s) leaves C partly written; it is
 *     counted in a word of the same static array (never in a context's
 *     counter) and read back by qt_noalloc_timeouts.                        */
#define QT_NOALLOC_MAX_BATCH 512
qt_status qt_zgemm_batch_noalloc(int n, int batch, char opA, const double* A, int64_t a_stride,
                                 char opB, const double* B, int64_t b_stride, const double* alpha,
                                 const double* beta, const double* D, int64_t d_stride, double* C,
                                 int64_t c_stride, int slices, void* stream);
/* Timeouts of qt_zgemm_batch_noalloc calls on the current device since the last
 * read: synchronises `stream`, stores the count in *count and clears it.  Call
 * it after the products' stream has finished; a non-zero count means those
 * results are incomplete.  No counterpart in the reference (see above).     */
qt_status qt_noalloc_timeouts(int* count, void* stream);

/* ---- GW / SCBA (device pointers: QT_FLAG_DEVICE_POINTERS required).
 * Energy-resolved arrays are [nk][nE][nx][nm*nm] complex128 column-major
 * slab-diagonal blocks, k slowest as the reference's (nm, nm, nx, nE, nk)
 * arrays; the energy grid E must be uniform (dE = E[1]-E[0]) and nE <= 2048
 * (zero-padded FFT length 4096).  V: nk nm x nm slab-diagonal Coulomb blocks,
 * one per momentum transfer q, or with QT_FLAG_V_PER_SLAB nk x nx blocks, one
 * per q and slab (the reference passes Vii/V1i per slab and q,
 * src/gw_mod.f90:84,597-600; only the diagonal block enters the per-slab W
 * restatement).  dev->nk k-points need H blocks per k (hii_kstride or
 * h1i_kstride non-zero).
 *
 * k-point grid and band (src/gw_mod.f90:466-555, 640-730): P at momentum
 * transfer q sums corr(G_k, G_kd) over k, Sigma at k sums conv(G_kd, W_q) over
 * q, with kd per direction = k - q + n_dir/2 (1-based, integer division)
 * wrapped once into range, k = kz + ky * nkz; the scales carry 1/nk.  ndiag >= 0
 * keeps only the elements |i - j| <= ndiag of P and Sigma (the reference's
 * ndiag), ndiag < 0 the full blocks.  qt_ctx_set_gw_grid sets nky x nkz and
 * ndiag for the context (default 1 x 1, full blocks); qt_gw_step and
 * qt_scba_solve use it when nky * nkz = dev->nk and take a one-direction grid
 * 1 x dev->nk when the context's grid is 1 x 1.  No counterpart: the
 * reference reads nky, nkz and ndiag as arguments of gw_ephoton_3d_ijs.    */
qt_status qt_ctx_set_gw_grid(qt_ctx* ctx, int nky, int nkz, int ndiag);

/* One evaluation of the SCBA map Sigma -> Sigma_new of gw_ephoton_3d_ijs
 * (src/gw_mod.f90:368-749 and :950-959): G by the batched RGF with
 * sigma_r/sigma_lesser (green_RGF_RS, :1131-1345), P by energy correlation of
 * the Re-zeroed G (:444-519), W = (I - V P^R)^-1 V and W^<> = W P^<> W^+ per
 * slab block (green_rgf_calc_w, called at :597, is absent from the
 * reference), Sigma by energy convolution (:646-698), Re/Im recombination,
 * symmetrisation (:698, :731-743) and the edge-block copy (:950-959).      */
qt_status qt_gw_step(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                     const qt_contacts* contacts, const double* V, double spindeg,
                     qt_precision prec, unsigned flags, const double* sigma_r,
                     const double* sigma_lesser, double* new_r, double* new_lesser,
                     double* new_greater);

/* Plain linear-mixing SCBA (src/gw_mod.f90:349-749) iterated until the
 * residual ||S_new - S||_F / ||S_new||_F over Sigma^< and Sigma^> is <= tol
 * or max_iter maps were evaluated (the reference has no convergence test and
 * runs a fixed niter).  sigma_* are the start values on input and the mixed
 * result on output; residuals [max_iter]; *iters = maps evaluated.
 * currents [max_iter][2] (host, may be NULL): the two columns of
 * Id_iteration.dat (src/gw_mod.f90:413-428), the left- and right-contact
 * currents (A) of each map's RGF, sum_E I(E) dE e0^2 spindeg / (2 pi hbar)
 * with the reference's constants e0 = 1.6022e-19 C, hbar = 1.0546e-34 J s.
 * The per-energy currents at any Sigma come from qt_rgf_solve with the
 * self-energies as sigma_r_ph / sigma_lesser_ph (tr, tre, bond_cur).      */
qt_status qt_scba_solve(qt_ctx* ctx, const qt_device* dev, const double* E, int nE,
                        const qt_contacts* contacts, const double* V, double spindeg,
                        double alpha, double tol, int max_iter, qt_precision prec,
                        unsigned flags, double* sigma_r, double* sigma_lesser,
                        double* sigma_greater, double* residuals, int* iters,
                        double* currents);

/* e-photon self-energy in the monochromatic approximation
 * (calc_sigma_ephoton_monochromatic_ext, src/gw_mod.f90:1075-1122), per energy e and
 * slab x:
 *   Sigma^<(e) = scale M_x [G^<(e - nop) + G^<(e + nop)] M_x, Sigma^> likewise,
 *   Sigma^R = i Im(Sigma^> - Sigma^<)/2,
 * scale = pre_fact * intensity / hw^2 and nop = floor(hw / dE) in the reference.
 *   M        [nx][nm*nm] interaction blocks (sum_i polarization(i) Pii(:,:,i,x))
 *   G_*      [nE + 2 nop][nx][nm*nm] with halo != 0 (nop energies from each neighbouring
 *            energy shard before and after, zero beyond the grid: src/gw_mod.f90:845-863),
 *            else [nE][nx][nm*nm] with zero beyond the ends
 *   sigma_*  [nE][nx][nm*nm] outputs
 * Device pointers (QT_FLAG_DEVICE_POINTERS), column-major complex128 blocks.      */
qt_status qt_ephoton_sigma(qt_ctx* ctx, int nm, int nx, int nE, int nop, int halo,
                           const double* M, const double* G_lesser, const double* G_greater,
                           double scale, qt_precision prec, unsigned flags, double* sigma_r,
                           double* sigma_lesser, double* sigma_greater);

/* ---- The SCBA map in stages, for ranks that share the energy grid.
 * With the context's grid of nk = nky * nkz k-points every array holds nk
 * k-blocks one after another (k slowest), each laid out as below, and the
 * polarisation / self-energy sum over k-pairs as qt_gw_step does; the band
 * is applied to blocks: P's in qt_gw_screened, Sigma's in qt_gw_sigma_post.
 * gw_ephoton_3d_ijs computes G on each rank's energies, moves G to (i, j)-major
 * order with an all-to-all (energies_to_ijs_2, src/gw_mod.f90:41-73), takes P
 * by energy correlations over the full grid on each rank's (i, j) elements,
 * moves P back to energies for W, W to (i, j) for Sigma, and Sigma back
 * (:452-456, 522-524, 636-638, 700-702).  These entry points are the compute
 * between those exchanges; qt_gw_step is the same sequence on one rank and
 * gives the same numbers.
 *
 * Series arrays hold nseries energy series of n points (the full energy grid),
 * energy-major: element (e, s) at 2*(e*nseries + s) doubles.  Block arrays hold
 * nm x nm column-major complex128 blocks back to back.  Device pointers only
 * (QT_FLAG_DEVICE_POINTERS); n <= 2048.                                     */

/* P^< = -i scale corr(G^<, G^>t), P^> = -i scale corr(G^>, G^<t),
 * P^R = -i scale [corr(G^<, conj G^R) + corr(G^R, G^<t)] with Re G zeroed
 * first (src/gw_mod.f90:444-446, 495-519).  G^<t / G^>t hold the transposed
 * element (j, i) of the same slab in the place of (i, j).  The reference's
 * scale is dE / (2 pi) * spindeg / nk.                                       */
qt_status qt_gw_polarization(qt_ctx* ctx, int n, int64_t nseries, const double* GR,
                             const double* GL, const double* GG, const double* GLt,
                             const double* GGt, double scale, double* PR, double* PL,
                             double* PG, unsigned flags);

/* W^R = (I - V P^R)^-1 V and W^{<,>} = W^R P^{<,>} W^R^+ for nblocks blocks
 * (the restatement of the absent green_rgf_calc_w, src/gw_mod.f90:597): nk
 * equal groups of blocks, group q with V block q (one group and one V block
 * for one k-point), P banded first when the context's ndiag >= 0.  Each W
 * may overwrite its own P (W^R over P^R, W^< over P^<, W^> over P^>), not
 * another one; the blocks are processed in chunks of about 8 GB of context
 * scratch.  QT_PREC_MIXED / QT_PREC_MIXED_FP64 take
 * the FP64-grade split products and refined inverses of the leads
 * (nm <= 384).  Synchronises.                                               */
qt_status qt_gw_screened(qt_ctx* ctx, int nm, int64_t nblocks, const double* V,
                         const double* PR, const double* PL, const double* PG, double* WR,
                         double* WL, double* WG, qt_precision prec, unsigned flags);

/* Sigma^< = i scale conv(G^<, W^<), Sigma^> = i scale conv(G^>, W^>),
 * Sigma^R = i scale [conv(G^<, W^R) + conv(G^R, W^<) + conv(G^R, W^R)], Re G
 * zeroed (src/gw_mod.f90:646-698); the reference's scale is dE / (2 pi) / nk.
 * Sigma^R is not yet recombined: see qt_gw_sigma_post.                      */
qt_status qt_gw_selfenergy(qt_ctx* ctx, int n, int64_t nseries, const double* GR,
                           const double* GL, const double* GG, const double* WR,
                           const double* WL, const double* WG, double scale, double* SR,
                           double* SL, double* SG, unsigned flags);

/* In place on [nk][nE][nx] blocks: the band (context's ndiag >= 0), then
 * Sigma^R <- Re Sigma^R + i Im(Sigma^> - Sigma^<)/2
 * (src/gw_mod.f90:698), S <- (S + S^T)/2 for all three (:731-743), and with
 * nx >= 5 the edge blocks 1,2 <- 3 and nx-1,nx <- nx-2 (:950-959).          */
qt_status qt_gw_sigma_post(qt_ctx* ctx, int nm, int nx, int nE, double* SR, double* SL,
                           double* SG, unsigned flags);

/* Batched energy correlation (mode 0) / convolution (mode 1) of corr1d2 /
 * conv1d2 (src/fft_mod.f90:58-168) on n-point series stored energy-major,
 * element (e, s) at 2*(e*nseries + s) doubles:
 *   mode 0: Z[m] = sum_e X[e] Y[e - (m - n/2)]
 *   mode 1: Z[e] = sum_m X[e - (m - n/2)] Y[m]          n <= 2048.          */
qt_status qt_corr_batch(qt_ctx* ctx, int n, int64_t nseries, const double* X, const double* Y,
                        double* Z, int mode, unsigned flags);

/* ---------------------------------------------------------------------------
 * Learned SCBA mixing: the multilayer perceptron that proposes the next
 * self-energy iterate.  No counterpart in the reference, whose SCBA loop mixes
 * linearly (src/gw_mod.f90:747-749).
 *
 * Network: n_in -> width -> ... -> width -> n_out with `depth` GELU hidden
 * layers; BF16 weights and activations, FP32 accumulation on the tensor cores,
 * FP32 master parameters, AdamW (beta1 0.9, beta2 0.999, eps 1e-8, weight decay
 * decoupled and applied to every parameter), loss = mean squared error over all
 * outputs.  Parameters are one flat FP32 array: for each layer l, W_l
 * (dout x din, row-major) followed by b_l (dout).
 * Inputs X [batch][n_in], targets T and outputs Y [batch][n_out], row-major
 * FP32; device pointers with QT_FLAG_DEVICE_POINTERS, host pointers otherwise.
 * ------------------------------------------------------------------------- */
typedef struct qt_mlp qt_mlp;

/* init_params: host array of qt_mlp_num_params floats, or NULL for
 * Glorot-uniform weights (seeded) and zero biases.  Runs on ctx's stream.   */
qt_status qt_mlp_create(qt_ctx* ctx, int n_in, int width, int depth, int n_out, int max_batch,
                        const float* init_params, uint64_t seed, qt_mlp** out);
qt_status qt_mlp_destroy(qt_mlp* net);
qt_status qt_mlp_num_params(const qt_mlp* net, int64_t* count);
qt_status qt_mlp_get_params(qt_mlp* net, float* host_params);
qt_status qt_mlp_set_params(qt_mlp* net, const float* host_params);
/* Y = net(X) */
qt_status qt_mlp_infer(qt_mlp* net, int batch, const float* X, float* Y, unsigned flags);
/* gradient of the loss at the current parameters (host output, flat like the
 * parameters) and the loss; no update                                      */
qt_status qt_mlp_grad(qt_mlp* net, int batch, const float* X, const float* T, float* grad_host,
                      double* loss, unsigned flags);
/* one AdamW step on the batch; loss (host, nullable) is the loss before the
 * step.  Asynchronous when loss is NULL and QT_FLAG_SYNC is not set.       */
qt_status qt_mlp_train_step(qt_mlp* net, int batch, const float* X, const float* T, float lr,
                            float weight_decay, double* loss, unsigned flags);

/* Mixing kernels (device pointers; QT_FLAG_SYNC synchronises).  Self-energies
 * are [nE][nx][nm*nm] complex128 column-major blocks; orbital o = l*nm + i.
 * No counterpart in the reference (linear mixing only).
 *
 * qt_mix_diag:     out[q][e][o] = Im X_q[e][l][i,i], q = 0 (XL), 1 (XG)
 * qt_mix_features: network input rows feats[o][2*nhist*64 + 2] from a ring
 *                  [h][q][e][o] of nhist (<= 3) diagonal residual series,
 *                  newest first: 64 Chebyshev coefficients per series
 *                  (Qt: [nE][64] projector) scaled by the newest pair's norm
 *                  and clamped to +-8,
 *                  then log10(residual)/8 and the orbital's log10 decay
 * qt_mix_apply:    out = S + a_ij R + b_ij (S - S_prev), a_ij = (a_i + a_j)/2,
 *                  b_ij likewise; row o of ab [norb][ncols] holds a_o (ncols 1,
 *                  b = 0) or (a_o, b_o) (ncols 2), clamped to [0, alpha_max]
 *                  and [beta_min, beta_max]; S_prev may be NULL; out may be S
 * qt_mix_gram:     G[i][j] = Re <XL_i, XL_j> + Re <XG_i, XG_j> (host k x k)
 * qt_mix_combine:  out = sum_i coef_i (X_i + alpha R_i)  (k <= 8 vectors)   */
qt_status qt_mix_diag(qt_ctx* ctx, int nE, int nx, int nm, const double* XL, const double* XG,
                      double* out, unsigned flags);
qt_status qt_mix_features(qt_ctx* ctx, int nE, int64_t norb, int nhist, const double* ring,
                          const double* Qt, double log_residual, float* feats, unsigned flags);
qt_status qt_mix_apply(qt_ctx* ctx, int nE, int nx, int nm, const float* ab, int ncols,
                       double alpha_max, double beta_min, double beta_max, const double* S,
                       const double* R, const double* S_prev, double* out, unsigned flags);
qt_status qt_mix_gram(qt_ctx* ctx, int64_t count, int k, const double* const* XL,
                      const double* const* XG, double* G_host);
qt_status qt_mix_combine(qt_ctx* ctx, int64_t count, int k, const double* coef,
                         const double* const* X, const double* const* R, double alpha,
                         double* out, unsigned flags);

#ifdef __cplusplus
}
#endif

#endif /* QT_RGF_H */
