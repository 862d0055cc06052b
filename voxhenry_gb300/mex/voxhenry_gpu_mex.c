/*
 * voxhenry_gpu_mex.c -- MATLAB / Octave gateway of libvhgpu.so (the GB300 solve path of VoxHenry).
 *
 * One MEX function with a command argument; the .m shims beside it give the reference's names and
 * argument lists (lse_matvect_mult.m, lse_sparse_precon_prepare.m, lse_sparse_precon_multiply.m,
 * pgmres.m, fpgmres.m) and shadow the reference's files when this folder is ahead of
 * src_lse_formation/ and src_iterative_solver/ on the path.  One file, so that the geometry and the
 * factor cached by one call are seen by the next (the reference keeps its factor in MATLAB globals,
 * src_lse_formation/lse_sparse_precon_prepare.m:2).
 *
 *   y = voxhenry_gpu_mex('matvec', JIn0, fN_all, Ae, z_real, z_imag, dx, idxS5)
 *         lse_matvect_mult.m:1 -- one product of the VIE operator on the device
 *   voxhenry_gpu_mex('precon_prepare', dx, z_real, z_imag, idxS, st_sparse_precon, Ae [, kind])
 *         lse_sparse_precon_prepare.m:1 -- kept until the factor is needed (below)
 *   y = voxhenry_gpu_mex('precon_multiply', JOut_full_in [, prectol])
 *         lse_sparse_precon_multiply.m:1
 *   [x, flag, relres, iter, resvec] = voxhenry_gpu_mex('gmres', b, restart, tol, maxit, flexible, x0,
 *         fN_all, Ae, z_real, z_imag, dx, idxS5 [, use_precon])
 *         pgmres.m:70 / fpgmres.m:58 with the operator of lse_matvect_mult and the prepared factor:
 *         the whole Krylov loop on the device (one call instead of one gateway call per iteration)
 *   voxhenry_gpu_mex('reset')   -- frees the cached handles
 *
 * Inputs follow the reference: complex double fN_all (2L x 2M x 2N x 7), real double sparse Ae (the
 * executer's Ae with the port rows removed), z_real (L x M x N) and z_imag ([] for normal conductors),
 * idxS5 / idxS as 1-based doubles.  Complex arrays are read in either layout: interleaved
 * (MATLAB R2018a and later, built with -R2018a, which defines MX_HAS_INTERLEAVED_COMPLEX) or split
 * real / imaginary parts (earlier MATLAB releases and Octave's mkoctfile --mex); the split layout is
 * interleaved into scratch memory around each call.
 *
 * The operator's geometry is cached by the data pointer and size of fN_all and the data pointer of
 * z_real (MATLAB's copy-on-write keeps them stable across the calls of one frequency,
 * VoxHenry_executer.m:287-290).  The executer prepares the preconditioner before the frequency's first
 * product, so lse_sparse_precon_prepare keeps (copies) its arguments and the factor is built on the
 * geometry that first needs it: the operator's (gmres) or a preconditioner-only geometry
 * (precon_multiply).  A failing call raises VoxHenryGPU:<status> with the library's message.
 *
 *   mex -R2018a voxhenry_gpu_mex.c -I<repo>/include -L<repo>/voxhenry_gb300 -lvhgpu
 *   mkoctfile --mex voxhenry_gpu_mex.c -I<repo>/include -L<repo>/voxhenry_gb300 -lvhgpu
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "voxhenry_gpu.h"

static vh_ctx* g_ctx = NULL;
static vh_geom* g_geom = NULL;        /* the operator's geometry (with the tensor) */
static const void* g_key_fN = NULL;   /* its cache key: fN_all's data and size, z_real's data */
static size_t g_key_n = 0;
static const void* g_key_z = NULL;

/* lse_sparse_precon_prepare's arguments (copies) */
static struct {
  int valid, L, M, N, has_prectol;
  double dx, st[6], prectol;
  vh_precon_kind kind;
  double *z_real, *z_imag;   /* L M N reals; 2 L M N interleaved or NULL */
  int64_t nv, nrow, ncol, *idxS, *jc, *ir;
  double* pr;
} g_prep;
static vh_geom* g_pc_geom = NULL;     /* preconditioner-only geometry (no tensor) */
static vh_precon* g_precon = NULL;    /* the factor, built on g_precon_on */
static vh_geom* g_precon_on = NULL;

static void free_prep(void) {
  free(g_prep.z_real);
  free(g_prep.z_imag);
  free(g_prep.idxS);
  free(g_prep.jc);
  free(g_prep.ir);
  free(g_prep.pr);
  memset(&g_prep, 0, sizeof g_prep);
}

static void drop_precon(void) {
  if (g_precon) vh_precon_destroy(g_precon);
  if (g_pc_geom) vh_geom_destroy(g_pc_geom);
  g_precon = NULL;
  g_precon_on = NULL;
  g_pc_geom = NULL;
}

static void release_all(void) {
  drop_precon();
  free_prep();
  if (g_geom) vh_geom_destroy(g_geom);
  if (g_ctx) vh_ctx_destroy(g_ctx);
  g_geom = NULL;
  g_ctx = NULL;
  g_key_fN = NULL;
  g_key_n = 0;
  g_key_z = NULL;
}

static void check(vh_status s) {
  if (s != VH_OK) {
    char id[64];
    const char* name = vh_status_string(s);
    strcpy(id, "VoxHenryGPU:");
    strncat(id, name ? name : "error", sizeof id - strlen(id) - 1);
    mexErrMsgIdAndTxt(id, "%s: %s", name ? name : "error", g_ctx ? vh_last_error(g_ctx) : "no context");
  }
}

static void ensure_ctx(void) {
  if (!g_ctx) {
    vh_status s = vh_ctx_create(0, &g_ctx);
    if (s != VH_OK) {
      g_ctx = NULL;
      mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_NO_DEVICE", "no CUDA device for the VoxHenry GPU path (%s)",
                        vh_status_string(s));
    }
    mexAtExit(release_all);
  }
}

/* ---- complex arrays in either layout ------------------------------------------------------------
 * A complex (or real, promoted) double array as interleaved (re, im) pairs: a view of the array's own
 * data when it is interleaved complex, else a copy (free with release_cplx). */
static const double* cplx_view(const mxArray* a, int* owned) {
  const size_t n = mxGetNumberOfElements(a);
  *owned = 0;
  if (!mxIsDouble(a)) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "expected a double array");
#ifdef MX_HAS_INTERLEAVED_COMPLEX
  if (mxIsComplex(a)) return (const double*)mxGetComplexDoubles(a);
  {
    const double* re = mxGetDoubles(a);
    double* out = (double*)mxMalloc(2 * n * sizeof(double) + 1);
    for (size_t i = 0; i < n; ++i) {
      out[2 * i] = re[i];
      out[2 * i + 1] = 0.0;
    }
    *owned = 1;
    return out;
  }
#else
  {
    const double* re = mxGetPr(a);
    const double* im = mxIsComplex(a) ? mxGetPi(a) : NULL;
    double* out = (double*)mxMalloc(2 * n * sizeof(double) + 1);
    for (size_t i = 0; i < n; ++i) {
      out[2 * i] = re[i];
      out[2 * i + 1] = im ? im[i] : 0.0;
    }
    *owned = 1;
    return out;
  }
#endif
}

static void release_cplx(const double* p, int owned) {
  if (owned) mxFree((void*)p);
}

/* an n x 1 complex output filled from interleaved pairs */
static mxArray* cplx_out(const double* v, size_t n) {
  mxArray* a = mxCreateDoubleMatrix((mwSize)n, 1, mxCOMPLEX);
#ifdef MX_HAS_INTERLEAVED_COMPLEX
  memcpy(mxGetComplexDoubles(a), v, 2 * n * sizeof(double));
#else
  {
    double* re = mxGetPr(a);
    double* im = mxGetPi(a);
    for (size_t i = 0; i < n; ++i) {
      re[i] = v[2 * i];
      im[i] = v[2 * i + 1];
    }
  }
#endif
  return a;
}

static double* real_data(const mxArray* a) {
#ifdef MX_HAS_INTERLEAVED_COMPLEX
  return mxGetDoubles(a);
#else
  return mxGetPr(a);
#endif
}

/* ---- geometry ----------------------------------------------------------------------------------- */
/* Ae (real sparse CSC, num_node x 5nv) as int64 column offsets and row indices (mxMalloc'd) */
static void csc_of(const mxArray* Ae, int64_t** jc, int64_t** ir, int64_t* ncol, int64_t* nrow) {
  if (!mxIsSparse(Ae) || mxIsComplex(Ae)) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "Ae must be real sparse");
  *ncol = (int64_t)mxGetN(Ae);
  *nrow = (int64_t)mxGetM(Ae);
  {
    const mwIndex* mjc = mxGetJc(Ae);
    const mwIndex* mir = mxGetIr(Ae);
    const int64_t nnz = (int64_t)mjc[*ncol];
    *jc = (int64_t*)mxMalloc((size_t)(*ncol + 1) * sizeof(int64_t));
    *ir = (int64_t*)mxMalloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    for (int64_t j = 0; j <= *ncol; ++j) (*jc)[j] = (int64_t)mjc[j];
    for (int64_t k = 0; k < nnz; ++k) (*ir)[k] = (int64_t)mir[k];
  }
}

/* the first nv entries of idxS5 (or all of idxS) as int64, 1-based (mxMalloc'd) */
static int64_t* idx_of(const mxArray* a, int64_t nv) {
  const double* d = real_data(a);
  int64_t* out = (int64_t*)mxMalloc((size_t)(nv > 0 ? nv : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < nv; ++i) out[i] = (int64_t)d[i];
  return out;
}

/* the operator's geometry for (fN_all, Ae, z_real, z_imag, dx, idxS5), cached */
static vh_geom* geometry_of(const mxArray* fN, const mxArray* Ae, const mxArray* zr, const mxArray* zi,
                            const mxArray* dx, const mxArray* idx) {
  const void* key = mxGetData(fN);
  const size_t keyn = mxGetNumberOfElements(fN);
  if (g_geom && key == g_key_fN && keyn == g_key_n && mxGetData(zr) == g_key_z) return g_geom;
  {
    const mwSize* d;
    int64_t *jc, *ir, ncol, nrow, nv, *idxS;
    const double *fn, *zim = NULL;
    int own_fn = 0, own_zi = 0;
    vh_status s;
    if (mxGetNumberOfDimensions(fN) != 4) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "fN_all must be 2L x 2M x 2N x 7");
    d = mxGetDimensions(fN);
    csc_of(Ae, &jc, &ir, &ncol, &nrow);
    nv = (int64_t)mxGetNumberOfElements(idx) / 5;
    if (5 * nv != ncol) {
      mxFree(jc);
      mxFree(ir);
      mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "Ae has %lld columns for %lld voxels", (long long)ncol,
                        (long long)nv);
    }
    idxS = idx_of(idx, nv);
    fn = cplx_view(fN, &own_fn);
    if (zi && !mxIsEmpty(zi)) zim = cplx_view(zi, &own_zi);
    if (g_precon && g_precon_on == g_geom) {   /* a factor built on the geometry being replaced */
      vh_precon_destroy(g_precon);
      g_precon = NULL;
      g_precon_on = NULL;
    }
    if (g_geom) vh_geom_destroy(g_geom);
    g_geom = NULL;
    s = vh_geom_create(g_ctx, (int)(d[0] / 2), (int)(d[1] / 2), (int)(d[2] / 2), mxGetScalar(dx), fn, nv, idxS, nrow,
                       jc, ir, real_data(Ae), real_data(zr), zim, 0, &g_geom);
    release_cplx(fn, own_fn);
    release_cplx(zim, own_zi);
    mxFree(idxS);
    mxFree(jc);
    mxFree(ir);
    check(s);
    g_key_fN = key;
    g_key_n = keyn;
    g_key_z = mxGetData(zr);
  }
  return g_geom;
}

static int64_t geom_n(vh_geom* g) {
  int64_t nc, nn, n;
  check(vh_geom_sizes(g, &nc, &nn, &n));
  return n;
}

static vh_precon_kind kind_of(const mxArray* a) {
  char name[64];
  if (!a) return VH_PRECON_SCHUR_INVERT;
  if (mxGetString(a, name, sizeof name) != 0) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "bad preconditioner type");
  if (!strcmp(name, "schur_invert")) return VH_PRECON_SCHUR_INVERT;
  if (!strcmp(name, "schur_approx")) return VH_PRECON_SCHUR_APPROX;
  if (!strcmp(name, "schur_gmres")) return VH_PRECON_SCHUR_GMRES;
  if (!strcmp(name, "no_precond")) return VH_PRECON_NONE;
  mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_UNSUPPORTED", "preconditioner '%s' is not provided", name);
  return VH_PRECON_NONE;
}

/* the prepared factor on geometry g (built there on first use) */
static vh_precon* precon_on(vh_geom* g) {
  if (!g_prep.valid) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "lse_sparse_precon_prepare has not been called");
  if (g_precon && g_precon_on == g) return g_precon;
  if (g_precon) vh_precon_destroy(g_precon);
  g_precon = NULL;
  g_precon_on = NULL;
  check(vh_precon_create(g, g_prep.kind, g_prep.st, 0, &g_precon));
  g_precon_on = g;
  if (g_prep.has_prectol) check(vh_precon_set_prectol(g_precon, g_prep.prectol));
  return g_precon;
}

/* the geometry a lone lse_sparse_precon_multiply applies the factor on: the operator's when the factor
 * lives there, else a preconditioner-only geometry built from the prepared arguments */
static vh_geom* precon_geometry(void) {
  if (g_geom && g_precon_on == g_geom) return g_geom;
  if (!g_pc_geom) {
    if (!g_prep.valid) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "lse_sparse_precon_prepare has not been called");
    check(vh_geom_create(g_ctx, g_prep.L, g_prep.M, g_prep.N, g_prep.dx, NULL, g_prep.nv, g_prep.idxS, g_prep.nrow,
                         g_prep.jc, g_prep.ir, g_prep.pr, g_prep.z_real, g_prep.z_imag, 0, &g_pc_geom));
  }
  return g_pc_geom;
}

/* ---- commands ----------------------------------------------------------------------------------- */
static void cmd_matvec(mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  /* JIn0, fN_all, Ae, z_real, z_imag, dx, idxS5 */
  vh_geom* g;
  int64_t n;
  const double* x;
  double* y;
  int own;
  if (nrhs < 7) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "matvec takes JIn0, fN_all, Ae, z_real, z_imag, dx, idxS5");
  g = geometry_of(prhs[1], prhs[2], prhs[3], prhs[4], prhs[5], prhs[6]);
  n = geom_n(g);
  if ((int64_t)mxGetNumberOfElements(prhs[0]) != n) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "JIn0 has the wrong length");
  x = cplx_view(prhs[0], &own);
  y = (double*)mxMalloc((size_t)n * 2 * sizeof(double));
  {
    vh_status s = vh_matvec(g, 1, x, y, NULL, NULL, VH_PREC_FP64);
    release_cplx(x, own);
    if (s != VH_OK) mxFree(y);
    check(s);
  }
  plhs[0] = cplx_out(y, (size_t)n);
  mxFree(y);
}

static void cmd_precon_prepare(int nrhs, const mxArray* prhs[]) {
  /* dx, z_real, z_imag, idxS, st_sparse_precon, Ae [, kind] */
  const mwSize* d;
  const double* st;
  int own;
  size_t lmn;
  int64_t *jc, *ir, *idx, nnz;
  if (nrhs < 6) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG",
                                  "precon_prepare takes dx, z_real, z_imag, idxS, st_sparse_precon, Ae [, kind]");
  if (mxGetNumberOfElements(prhs[4]) != 3) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "st_sparse_precon has 3 entries");
  drop_precon();
  free_prep();
  g_prep.kind = kind_of(nrhs > 6 ? prhs[6] : NULL);
  g_prep.dx = mxGetScalar(prhs[0]);
  d = mxGetDimensions(prhs[1]);
  g_prep.L = (int)d[0];
  g_prep.M = mxGetNumberOfDimensions(prhs[1]) > 1 ? (int)d[1] : 1;
  g_prep.N = mxGetNumberOfDimensions(prhs[1]) > 2 ? (int)d[2] : 1;
  lmn = mxGetNumberOfElements(prhs[1]);
  g_prep.z_real = (double*)malloc(lmn * sizeof(double) + 1);
  memcpy(g_prep.z_real, real_data(prhs[1]), lmn * sizeof(double));
  if (!mxIsEmpty(prhs[2])) {
    const double* zi = cplx_view(prhs[2], &own);
    g_prep.z_imag = (double*)malloc(2 * lmn * sizeof(double) + 1);
    memcpy(g_prep.z_imag, zi, 2 * lmn * sizeof(double));
    release_cplx(zi, own);
  }
  g_prep.nv = (int64_t)mxGetNumberOfElements(prhs[3]);
  idx = idx_of(prhs[3], g_prep.nv);
  g_prep.idxS = (int64_t*)malloc((size_t)(g_prep.nv > 0 ? g_prep.nv : 1) * sizeof(int64_t));
  memcpy(g_prep.idxS, idx, (size_t)g_prep.nv * sizeof(int64_t));
  mxFree(idx);
  csc_of(prhs[5], &jc, &ir, &g_prep.ncol, &g_prep.nrow);
  nnz = jc[g_prep.ncol];
  g_prep.jc = (int64_t*)malloc((size_t)(g_prep.ncol + 1) * sizeof(int64_t));
  g_prep.ir = (int64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
  g_prep.pr = (double*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(double));
  memcpy(g_prep.jc, jc, (size_t)(g_prep.ncol + 1) * sizeof(int64_t));
  memcpy(g_prep.ir, ir, (size_t)nnz * sizeof(int64_t));
  memcpy(g_prep.pr, real_data(prhs[5]), (size_t)nnz * sizeof(double));
  mxFree(jc);
  mxFree(ir);
  st = cplx_view(prhs[4], &own);
  memcpy(g_prep.st, st, 6 * sizeof(double));
  release_cplx(st, own);
  g_prep.valid = 1;
}

static void cmd_precon_multiply(mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  int64_t n;
  const double* x;
  double* y;
  int own;
  vh_geom* g;
  vh_precon* pc;
  if (nrhs < 1) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "precon_multiply takes JOut_full_in [, prectol]");
  if (nrhs > 1 && !mxIsEmpty(prhs[1])) {
    g_prep.prectol = mxGetScalar(prhs[1]);
    g_prep.has_prectol = 1;
  }
  g = precon_geometry();
  pc = precon_on(g);
  if (g_prep.has_prectol) check(vh_precon_set_prectol(pc, g_prep.prectol));
  n = geom_n(g);
  if ((int64_t)mxGetNumberOfElements(prhs[0]) != n) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "wrong length");
  x = cplx_view(prhs[0], &own);
  y = (double*)mxMalloc((size_t)n * 2 * sizeof(double));
  {
    vh_status s = vh_precon_apply(g, 1, &pc, x, y);
    release_cplx(x, own);
    if (s != VH_OK) mxFree(y);
    check(s);
  }
  plhs[0] = cplx_out(y, (size_t)n);
  mxFree(y);
}

static void cmd_gmres(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  /* b, restart, tol, maxit, flexible, x0, fN_all, Ae, z_real, z_imag, dx, idxS5 [, use_precon] */
  vh_geom* g;
  int64_t n;
  int restart, maxit, flexible, use_pc, flag = 1, iter[2] = {0, 0}, nres = 0, rlen;
  double tol, relres = 0.0, *x, *resvec;
  const double *b, *x0 = NULL;
  int own_b, own_x0 = 0;
  vh_precon* pcs[1];
  if (nrhs < 12) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG",
                                   "gmres takes b, restart, tol, maxit, flexible, x0, fN_all, Ae, z_real, z_imag, dx, idxS5");
  g = geometry_of(prhs[6], prhs[7], prhs[8], prhs[9], prhs[10], prhs[11]);
  n = geom_n(g);
  restart = (int)mxGetScalar(prhs[1]);
  tol = mxGetScalar(prhs[2]);
  maxit = (int)mxGetScalar(prhs[3]);
  flexible = (int)mxGetScalar(prhs[4]);
  use_pc = nrhs > 12 ? (int)mxGetScalar(prhs[12]) : 1;
  if (restart < 1 || maxit < 1) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "restart and maxit must be positive");
  if ((int64_t)mxGetNumberOfElements(prhs[0]) != n) mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "b has the wrong length");
  pcs[0] = use_pc ? precon_on(g) : NULL;
  b = cplx_view(prhs[0], &own_b);
  if (!mxIsEmpty(prhs[5])) {
    if ((int64_t)mxGetNumberOfElements(prhs[5]) != n) {
      release_cplx(b, own_b);
      mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "x0 has the wrong length");
    }
    x0 = cplx_view(prhs[5], &own_x0);
  }
  rlen = restart * maxit + 1;
  x = (double*)mxMalloc((size_t)n * 2 * sizeof(double));
  resvec = (double*)mxMalloc((size_t)rlen * sizeof(double));
  {
    vh_status s = vh_gmres_x0(g, 1, use_pc ? pcs : NULL, b, NULL, NULL, restart, &tol, maxit, flexible, VH_PREC_FP64,
                              x0, x, &flag, &relres, iter, resvec, rlen, &nres);
    release_cplx(b, own_b);
    release_cplx(x0, own_x0);
    if (s != VH_OK) {
      mxFree(x);
      mxFree(resvec);
    }
    check(s);
  }
  plhs[0] = cplx_out(x, (size_t)n);
  if (nlhs > 1) plhs[1] = mxCreateDoubleScalar((double)flag);
  if (nlhs > 2) plhs[2] = mxCreateDoubleScalar(relres);
  if (nlhs > 3) {   /* iter = [inner iterations of the last cycle, outer cycles] (pgmres.m:178) */
    plhs[3] = mxCreateDoubleMatrix(1, 2, mxREAL);
    real_data(plhs[3])[0] = (double)iter[0];
    real_data(plhs[3])[1] = (double)iter[1];
  }
  if (nlhs > 4) {
    const int k = nres < rlen ? nres : rlen;
    plhs[4] = mxCreateDoubleMatrix((mwSize)k, 1, mxREAL);
    memcpy(real_data(plhs[4]), resvec, (size_t)k * sizeof(double));
  }
  mxFree(x);
  mxFree(resvec);
}

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  char cmd[32];
  if (nrhs < 1 || !mxIsChar(prhs[0]) || mxGetString(prhs[0], cmd, sizeof cmd) != 0)
    mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "first argument: a command string");
  if (!strcmp(cmd, "reset")) {
    release_all();
    return;
  }
  ensure_ctx();
  if (!strcmp(cmd, "matvec"))
    cmd_matvec(plhs, nrhs - 1, prhs + 1);
  else if (!strcmp(cmd, "precon_prepare"))
    cmd_precon_prepare(nrhs - 1, prhs + 1);
  else if (!strcmp(cmd, "precon_multiply"))
    cmd_precon_multiply(plhs, nrhs - 1, prhs + 1);
  else if (!strcmp(cmd, "gmres"))
    cmd_gmres(nlhs, plhs, nrhs - 1, prhs + 1);
  else
    mexErrMsgIdAndTxt("VoxHenryGPU:VH_ERR_BAD_ARG", "unknown command '%s'", cmd);
}
