/*
 * voxhenry_gpu.h -- C ABI of the GB300 (sm_103a) VoxHenry solve-path library (libvhgpu.so).
 *
 * The library replaces the MATLAB/Octave hot path of VoxHenry:
 *   lse_matvect_mult            src_lse_formation/lse_matvect_mult.m:1
 *   lse_sparse_precon_prepare   src_lse_formation/lse_sparse_precon_prepare.m:1
 *   lse_sparse_precon_multiply  src_lse_formation/lse_sparse_precon_multiply.m:1
 *   pgmres / fpgmres            src_iterative_solver/pgmres.m:70, fpgmres.m:58
 * Conventions (as in the reference):
 *   - complex values are interleaved (re, im) doubles;
 *   - 3-D grids are column-major (x fastest), voxel indices 1-based (idxS);
 *   - the incidence matrix Ae (num_node x 5*nv, port rows already removed, the
 *     "Ar" of the executer) is passed in CSC form with 0-based row indices.
 * Every call returns a vh_status; vh_last_error() gives the text of the last failure
 * on a context.  Host pointers are borrowed for the duration of the call.
 * A context owns one CUDA stream; calls on one context must not overlap.
 * Handles may be destroyed in any order: a geometry keeps its context, and a preconditioner its
 * geometry, until it is destroyed itself.
 */
#ifndef VOXHENRY_GPU_H
#define VOXHENRY_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum vh_status {
  VH_OK = 0,
  VH_ERR_BAD_ARG = 1,
  VH_ERR_OOM = 2,
  VH_ERR_UNSUPPORTED = 3,
  VH_ERR_TIMEOUT = 4,   /* a device wait gave up (the Toeplitz z-pass's tensor copies); products NaN */
  VH_ERR_NOT_CONVERGED = 5,
  VH_ERR_CUDA = 6,
  VH_ERR_NO_DEVICE = 7
} vh_status;

/* arithmetic of the FFT convolution: complex128, or complex64 with fp32 accumulation */
/* VH_PREC_DF (vh_matvec / vh_matvec_device only): the FFT passes and the tensor products in
 * double-float (pairs of floats, ~48 significant bits, relative error ~1e-13) on GB300's FP32 pipes,
 * the spectra stored as pairs between the passes; no counterpart in the reference.  Grids whose
 * padded x or y length is not 256, 512 or 1024, whose z length has no register pass, or whose tensor
 * spectrum is not real/imaginary per component, get the complex128 product instead.  The
 * mixed-precision solver forms its refinement residual with it.                                   */
typedef enum vh_prec { VH_PREC_FP64 = 0, VH_PREC_FP32 = 1, VH_PREC_DF = 2 } vh_prec;

/* preconditioner kinds of lse_sparse_precon_prepare.m:5,71,83,90 ('schur_invert_original' is not provided) */
typedef enum vh_precon_kind {
  VH_PRECON_NONE = 0,            /* 'no_precond' */
  VH_PRECON_SCHUR_INVERT = 1,    /* 'schur_invert' : exact Schur complement, sparse Cholesky in FP64 */
  VH_PRECON_SCHUR_INVERT_DF = 2, /* 'schur_invert' with the factor and its triangular solves in double-float
                                    (FP32 pairs, ~48 significant bits, on GB300's FP32 pipes); no counterpart
                                    in the reference.  For the mixed-precision solver (VH_PREC_FP32), whose FP64
                                    residuals set the accuracy; FP64 solves to 1e-12 want VH_PRECON_SCHUR_INVERT */
  VH_PRECON_SCHUR_APPROX = 3,    /* 'schur_approx' (lse_sparse_precon_prepare.m:71-81, multiply.m:48-58): S^-1
                                    replaced by W Ae diag(A_inv)^-1 Ae^T W, W = diag(1 / sum_k |Ae(:,k)|); no factor */
  VH_PRECON_SCHUR_GMRES = 4      /* 'schur_gmres' (prepare.m:83-88, multiply.m:26-46): S^-1 applied by an inner
                                    restarted GMRES on S = Ae diag(A_inv) Ae^T with the Jacobi preconditioner
                                    diag(S), restart min(100, num_curr - 1), at most 10 cycles, tolerance prectol
                                    (vh_precon_set_prectol; 0.1 as VoxHenry_executer.m:38).  The apply is not a
                                    fixed linear operator: use it with flexible GMRES (VoxHenry_executer.m:294-297);
                                    the mixed-precision solver rejects it. */
} vh_precon_kind;

typedef struct vh_ctx vh_ctx;
typedef struct vh_geom vh_geom;
typedef struct vh_precon vh_precon;

/* ---- context ----------------------------------------------------------------------------- */
int vh_version(void);
const char* vh_status_string(vh_status s);
vh_status vh_ctx_create(int device, vh_ctx** out);
void vh_ctx_destroy(vh_ctx* ctx);
const char* vh_last_error(const vh_ctx* ctx);
vh_status vh_ctx_synchronize(vh_ctx* ctx);
/* device memory of the context's block cache (no counterpart in the reference): solver buffers and
 * factors are drawn from a per-context cache instead of cudaMalloc / cudaFree per call (both cost
 * milliseconds at these sizes and synchronise the device).  vh_ctx_memory: bytes handed out and bytes
 * cached; vh_ctx_trim: waits for the context's stream and frees the cached blocks (a server hands them
 * back before another context needs the memory).                                                   */
vh_status vh_ctx_memory(vh_ctx* ctx, int64_t* in_use, int64_t* cached);
vh_status vh_ctx_trim(vh_ctx* ctx);

/* ---- geometry: the fixed arguments of lse_matvect_mult (lse_matvect_mult.m:1) ------------------
 * fN_all      : circulant tensor spectrum, complex (2L, 2M, 2N, 7) column-major.  The drop-in passes
 *               the per-frequency fN_all = (j w mu) fN_all2 (VoxHenry_executer.m:266); the batched
 *               solver passes fN_all2 and a per-RHS scale j w mu.
 * idxS        : nv sorted 1-based linear indices of non-empty voxels (pre_define_structure_params.m:6-14);
 *               idxS5 of the reference is [idxS; idxS+LMN; ... ; idxS+4LMN].
 * Ae          : num_node x 5nv CSC (jc: 5nv+1 offsets, ir: 0-based rows, pr: values).
 * z_real      : (L,M,N) real; z_imag : (L,M,N) complex or NULL (VoxHenry_executer.m:231-259).
 * want_fp32   : also keep a complex64 copy of the tensor for VH_PREC_FP32 products.            */
vh_status vh_geom_create(vh_ctx* ctx, int L, int M, int N, double dx, const double* fN_all, int64_t nv,
                         const int64_t* idxS, int64_t num_node, const int64_t* Ae_jc, const int64_t* Ae_ir,
                         const double* Ae_pr, const double* z_real, const double* z_imag, int want_fp32,
                         vh_geom** out);
/* same, with the circulant tensor generated on the device (lse_generate_circulant_tensor(dx, 1, L, M, N, 0),
 * lse_generate_circulant_tensor.m:1; the batched-solver form fN_all2 of VoxHenry_executer.m:141).
 * st_sparse_precon (out, may be NULL): the 3 complex self terms st_sparse_precon2.              */
vh_status vh_geom_create_generated(vh_ctx* ctx, int L, int M, int N, double dx, int64_t nv, const int64_t* idxS,
                                   int64_t num_node, const int64_t* Ae_jc, const int64_t* Ae_ir, const double* Ae_pr,
                                   const double* z_real, const double* z_imag, int want_fp32, double* st_sparse_precon,
                                   vh_geom** out);
void vh_geom_destroy(vh_geom* g);
/* sizes: n_curr = 5 nv, n_node = rows of Ae, n = n_curr + n_node */
vh_status vh_geom_sizes(const vh_geom* g, int64_t* n_curr, int64_t* n_node, int64_t* n);
/* replaces z (per-voxel) in slot `slot` (0 = the z given at creation).  Superconductors have an
 * omega-dependent z; one slot per frequency.  z_imag may be NULL. */
vh_status vh_geom_set_z(vh_geom* g, int slot, const double* z_real, const double* z_imag);

/* ---- matvec: JOut_full = lse_matvect_mult(JIn0, ...) for B right-hand sides ---------------------
 * x, y   : HOST arrays, B x n complex (RHS b at offset b*n).
 * scale  : B complex factors multiplying the tensor (NULL: all 1, the drop-in form).
 * zslot  : B slot numbers (NULL: slot 0 for all).                                                */
vh_status vh_matvec(vh_geom* g, int B, const double* x, double* y, const double* scale, const int* zslot,
                    vh_prec prec);
/* same with DEVICE pointers, enqueued on the context stream (no synchronisation) */
vh_status vh_matvec_device(vh_geom* g, int B, const void* x_dev, void* y_dev, const void* scale_dev,
                           const int* zslot, vh_prec prec);

/* ---- autotuning of the FFT convolution (no counterpart in the reference) -----------------------
 * vh_conv_tune times the launch choices of the geometry's FFT convolution at precision `prec` for a
 * batch of B right-hand sides with CUDA events on the context stream (one warm-up and the best of
 * two products each; inputs are a constant pattern, the timing does not depend on the values),
 * keeps the fastest in the geometry and returns it: y_variant (1 the register y-pass for padded y
 * lengths 256, 512, 1024; 2 the shared-memory Stockham pass; 3 the register y-pass over 64-byte row
 * segments), z_variant (1 the two-lane register
 * z-pass; 2 one thread per column, for padded z lengths up to 32; 3, complex64 and double-float, the
 * direct Toeplitz convolution along z for voxel boxes up to 16 rows high), max_rhs (right-hand sides per
 * launch sequence; 0: the whole batch), x_variant (complex64: 1 one warp per line for padded x lengths
 * 256, 512, 1024, 2 the shared-memory x passes), and its milliseconds per RHS-matvec.
 * vh_conv_set_tuning sets a choice without timing (a cached one); zeros restore the automatic
 * choices (complex64: warp-per-line x passes where they apply, the Toeplitz z-pass for voxel boxes up
 * to 16 rows, the register y-pass over 64-byte rows).  The products of every
 * choice agree within the precision's rounding.                                                     */
vh_status vh_conv_tune(vh_geom* g, vh_prec prec, int B, int* y_variant, int* z_variant, int* max_rhs,
                       int* x_variant, double* ms_per_rhs);
vh_status vh_conv_set_tuning(vh_geom* g, vh_prec prec, int y_variant, int z_variant, int max_rhs, int x_variant);

/* ---- allocation-free matvec (no counterpart in the reference) -----------------------------------
 * The operator of vh_matvec_device, same arguments and results for VH_PREC_FP64 and VH_PREC_FP32,
 * enqueued on the context stream, but the call allocates no device memory (no cudaMalloc / cudaFree,
 * no allocating library routine).  VH_PREC_DF is rejected with VH_ERR_BAD_ARG: its first product
 * builds a pair copy of the tensor, an allocation.
 * For callers that cannot allocate at call time: a host whose device memory is all handed to its own
 * pool allocator (a framework's caching allocator under a memory cap), and a host whose solve loop
 * must not stall, since cudaMalloc / cudaFree synchronise the whole device and so serialise the work
 * of its other streams.
 *   - FFT scratch: one fixed device array of VH_MATVEC_NOALLOC_SCRATCH_BYTES per device, shared by
 *     every context on that device.  The right-hand sides are processed in groups that fit it (at
 *     most 64 per group); a grid whose single right-hand side needs more (30 L M N complex values of
 *     the precision) is rejected with VH_ERR_UNSUPPORTED.  Nothing in it needs to start at zero.
 *   - Calls whose GPU work overlaps (streams of different contexts on one device) race on that
 *     scratch: order them on the device (one context, or events between the streams).
 *   - The first call on a device does the set-up (it looks up the scratch array's device address and
 *     fills a table of unit scales, then synchronises the context stream); make that first call
 *     before any stream capture.  The addresses are kept for the life of the process: do not use the
 *     library across a cudaDeviceReset (or a reset of the primary context).
 *   - zslot: as vh_matvec_device (NULL: slot 0); every slot named must already be set.           */
#define VH_MATVEC_NOALLOC_SCRATCH_BYTES (16u << 20)
vh_status vh_matvec_device_noalloc(vh_geom* g, int B, const void* x_dev, void* y_dev, const void* scale_dev,
                                   const int* zslot, vh_prec prec);

/* ---- preconditioner: lse_sparse_precon_prepare(dx, z_real, z_imag, idxS, st_sparse_precon, ..., Ae)
 *      (lse_sparse_precon_prepare.m:1).  A geometry created with fN_all == NULL serves a
 *      preconditioner-only caller.  st_sparse_precon: 3 complex self terms (already multiplied by
 *      j w mu, VoxHenry_executer.m:267); z is taken from slot `zslot` of the geometry (dx too).
 *      The factor of the Schur complement is built on the device and kept in the handle (the
 *      reference keeps it in MATLAB globals, lse_sparse_precon_prepare.m:2).                    */
vh_status vh_precon_create(vh_geom* g, vh_precon_kind kind, const double* st_sparse_precon, int zslot,
                           vh_precon** out);
/* nfreq preconditioners at once (one per frequency), factored by one batched launch sequence:
 * st_sparse_precon: nfreq x 3 complex; zslot: nfreq slots (NULL: slot 0); out: nfreq handles.   */
vh_status vh_precon_create_batch(vh_geom* g, vh_precon_kind kind, int nfreq, const double* st_sparse_precon,
                                 const int* zslot, vh_precon** out);
void vh_precon_destroy(vh_precon* p);
/* 'schur_gmres': the `prectol` argument of lse_sparse_precon_multiply.m:1 (default 0.1), and the inner GMRES
 * iterations summed over every apply of this handle so far (the reference prints them, multiply.m:44). */
vh_status vh_precon_set_prectol(vh_precon* p, double prectol);
vh_status vh_precon_inner_iterations(const vh_precon* p, int64_t* total);
/* factor statistics: entries of L, factorisation flops, fronts, largest front order */
vh_status vh_precon_stats(const vh_precon* p, int64_t* nnz_factor, double* flops, int* nfronts, int* max_front);
/* host-only symbolic analysis of S = Ae diag Ae^T (no device needed): same statistics plus the bytes of
 * one frequency's factor storage -- used to admit jobs by device-memory footprint. */
vh_status vh_schur_analyze(int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t num_node,
                           const int64_t* Ae_jc, const int64_t* Ae_ir, const double* Ae_pr, int64_t* nnz_factor,
                           double* flops, int* nfronts, int* max_front, int64_t* factor_bytes);

/* ---- JOut_full_out = lse_sparse_precon_multiply(JOut_full_in, Ae, ...) (lse_sparse_precon_multiply.m:1)
 *      for B right-hand sides; RHS b uses pcs[b] (all of one kind).  x, y: HOST, B x n complex.   */
vh_status vh_precon_apply(vh_geom* g, int B, vh_precon* const* pcs, const double* x, double* y);
vh_status vh_precon_apply_device(vh_geom* g, int B, vh_precon* const* pcs, const void* x_dev, void* y_dev);

/* ---- [x,flag,relres,iter,resvec] = pgmres(A, b, restart, tol, maxit, L1)   (pgmres.m:70)
 *      or fpgmres(A, b, restart, tol, maxit, R1)                             (fpgmres.m:58)
 *      for B right-hand sides at once, A = lse_matvect_mult of geometry g with per-RHS scale/zslot,
 *      the preconditioner pcs[b] (NULL: none) on the left (flexible = 0) or right (flexible = 1).
 *      x0 = 0 (vh_gmres_x0 below takes one).  b, x: HOST B x n complex.  tol: B values.  Outputs per RHS: flag (0 converged),
 *      relres = |b - A x| / |b|, iter = [inner iterations of the last cycle, outer cycles] (2 ints),
 *      resvec (first resvec_len entries, row b at b*resvec_len), nres = its full length.
 *      prec = VH_PREC_FP32: mixed precision -- FP64 iterative refinement around left-preconditioned
 *      GMRES whose FFT matvec runs in complex64, refined until the residual |b - A x| meets tol: it is
 *      formed in FP64 after the first refinement step and then updated, r <- r - A d, with the complex64
 *      product of each (small) correction d, which keeps it within ~1e-6 |A d| (~1e-11 |b| at tol 1e-9)
 *      of the FP64 residual.  iter then counts inner iterations / cycles summed over refinement steps;
 *      resvec holds that relative residual after each step, relres its last value.  The inner
 *      GMRES keeps its Krylov basis in complex128 and runs its Gram-Schmidt sums in double-float.  */
vh_status vh_gmres(vh_geom* g, int B, vh_precon* const* pcs, const double* b, const double* scale, const int* zslot,
                   int restart, const double* tol, int maxit, int flexible, vh_prec prec, double* x, int* flag,
                   double* relres, int* iter, double* resvec, int resvec_len, int* nres);
/* same with b and x in DEVICE memory (B x n complex); returns after the solve has finished */
vh_status vh_gmres_device(vh_geom* g, int B, vh_precon* const* pcs, const void* b_dev, const double* scale,
                          const int* zslot, int restart, const double* tol, int maxit, int flexible, vh_prec prec,
                          void* x_dev, int* flag, double* relres, int* iter, double* resvec, int resvec_len, int* nres);
/* [x,flag,relres,iter,resvec] = pgmres(A, b, restart, tol, maxit, L1, [], [], [], x0)   (pgmres.m:70)
 * with an initial guess: as vh_gmres / vh_gmres_device, starting from x0 (B x n complex, HOST for
 * vh_gmres_x0, DEVICE for vh_gmres_device_x0; NULL: zero).  The first residual is b - A x0 (pgmres.m:111-113);
 * the mixed-precision solver forms it with the double-float product and refines from x0.             */
vh_status vh_gmres_x0(vh_geom* g, int B, vh_precon* const* pcs, const double* b, const double* scale, const int* zslot,
                      int restart, const double* tol, int maxit, int flexible, vh_prec prec, const double* x0,
                      double* x, int* flag, double* relres, int* iter, double* resvec, int resvec_len, int* nres);
vh_status vh_gmres_device_x0(vh_geom* g, int B, vh_precon* const* pcs, const void* b_dev, const double* scale,
                             const int* zslot, int restart, const double* tol, int maxit, int flexible, vh_prec prec,
                             const void* x0_dev, void* x_dev, int* flag, double* relres, int* iter, double* resvec,
                             int resvec_len, int* nres);

/* ---- instrumentation (no counterpart in the reference, which times with tic/toc) --------------
 * vh_ctx_stream: the CUDA stream (cudaStream_t) all work of the context is enqueued on.
 * vh_ctx_profile: enable/disable per-section CUDA-event timing (clears recorded sections).
 * vh_ctx_profile_read: milliseconds, call counts and work units (RHS) per section since the last read/enable:
 *   0 FFT convolution complex128, 1 FFT convolution complex64, 2 Ae/Ae^T products of the matvec,
 *   3 Schur factorisation, 4 preconditioner apply, 5 Krylov vector work, 6 tensor generation.
 * vh_launch_count: kernels launched by the library since it was loaded.                       */
void* vh_ctx_stream(vh_ctx* ctx);
vh_status vh_ctx_profile(vh_ctx* ctx, int enable);
vh_status vh_ctx_profile_read(vh_ctx* ctx, double* ms, int64_t* calls, int64_t* units, int nsec);
int64_t vh_launch_count(void);

/* ---- setup: the inputs of the solve path --------------------------------------------------------
 * [all_panels_ids, num_nodes] = lse_generate_panelIDs(idxS, L, M, N)   (lse_generate_panelIDs.m:1)
 *   all_panels_ids: nv x 6 column-major, 1-based node ids (-x,+x,-y,+y,-z,+z); no device needed. */
vh_status vh_panel_ids(int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t* all_panels_ids,
                       int64_t* num_nodes);
/* Ae = lse_compute_Ae_matrix(idxS, all_panels_ids, num_nodes) (lse_compute_Ae_matrix.m:1) as CSC:
 *   jc: 5nv+1, ir (0-based rows) and pr: 16 nv entries each; no device needed.                  */
vh_status vh_incidence(int64_t nv, const int64_t* all_panels_ids, int64_t* Ae_jc, int64_t* Ae_ir, double* Ae_pr);
/* Both of the above on the context's device, in one call (the per-request setup of a serving loop):
 *   all_panels_ids and num_nodes as vh_panel_ids; Ae_jc/Ae_ir/Ae_pr as vh_incidence, or all three NULL
 *   to skip Ae.  Host buffers; ids are built by prefix sums along each axis's scan order and equal the
 *   sequential numbering of lse_generate_panelIDs.m:25-172 exactly.  Grids up to 2^31 cells.       */
vh_status vh_setup_device(vh_ctx* ctx, int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t* all_panels_ids,
                          int64_t* num_nodes, int64_t* Ae_jc, int64_t* Ae_ir, double* Ae_pr);
/* [fN_all, st_sparse_precon] = lse_generate_circulant_tensor(dx, 1, L, M, N, 0)
 *   (lse_generate_circulant_tensor.m:1), computed on the device; fN_all (HOST, may be NULL):
 *   complex (2L, 2M, 2N, 7) column-major; st_sparse_precon (HOST, may be NULL): 3 complex.       */
vh_status vh_circulant_tensor(vh_ctx* ctx, int L, int M, int N, double dx, double* fN_all, double* st_sparse_precon);

/* ---- post-processing of the currents (src_post_process) -----------------------------------------
 * [Jx,Jy,Jz,J2d,J3d] grids of post_obtain_curr_coefs_on_grid(x, Mc) (post_obtain_curr_coefs_on_grid.m:1):
 *   x: HOST, B solutions (complex, leading dimension ldx >= 5 nv, current coefficients first);
 *   grids: HOST, B x 5 x (L M N) complex, column-major grids, zero outside the voxels; scattered on
 *   the device.  idxS: the nv 1-based voxel indices (pre_define_structure_params.m:6-14).        */
vh_status vh_currents_on_grid(vh_ctx* ctx, int L, int M, int N, int64_t nv, const int64_t* idxS, int B,
                              const double* x, int64_t ldx, double* grids);
/* y = A x for a real CSC matrix A (nrows x ncols, 0-based ir) and B complex HOST vectors (leading
 * dimensions ldx, ldy), on the device: the node currents -Ae_only_leaving x + Ae_only_entering_bndry x
 * of post_obtain_currs_on_nodes.m:7-9 (one product with the difference matrix).                */
vh_status vh_sparse_matvec(vh_ctx* ctx, int64_t nrows, int64_t ncols, const int64_t* jc, const int64_t* ir,
                           const double* pr, int B, const double* x, int64_t ldx, double* y, int64_t ldy);

#ifdef __cplusplus
}
#endif
#endif /* VOXHENRY_GPU_H */
