/* A host-only implementation of the MEX API subset in mex.h (test infrastructure): dense double
 * arrays (real or complex, in the layout the build selects), real sparse CSC matrices and strings,
 * plus stub_* entry points through which a test builds arguments, calls mexFunction and reads the
 * results.  mexErrMsgIdAndTxt returns to stub_call (longjmp) with the identifier and text. */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

struct mxArray_tag {
  int kind;   /* 0 dense double, 1 char, 2 sparse */
  int cplx;
  mwSize ndim, dims[8];
  size_t numel;
  double *re, *im;   /* split layout (im NULL for real) */
  double* ri;        /* interleaved layout (complex only) */
  mwIndex *jc, *ir;
  char* str;
};

static jmp_buf g_jmp;
static char g_err[1024];
static void (*g_atexit)(void) = NULL;

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  va_list ap;
  int k = snprintf(g_err, sizeof g_err, "%s|", id);
  va_start(ap, fmt);
  vsnprintf(g_err + k, sizeof g_err - (size_t)k, fmt, ap);
  va_end(ap);
  longjmp(g_jmp, 1);
}
int mexAtExit(void (*fn)(void)) {
  g_atexit = fn;
  return 0;
}
void* mxMalloc(size_t n) { return malloc(n ? n : 1); }
void mxFree(void* p) { free(p); }

size_t mxGetNumberOfElements(const mxArray* a) { return a->numel; }
mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->ndim; }
const mwSize* mxGetDimensions(const mxArray* a) { return a->dims; }
size_t mxGetM(const mxArray* a) { return a->dims[0]; }
size_t mxGetN(const mxArray* a) {
  size_t n = 1;
  for (mwSize k = 1; k < a->ndim; ++k) n *= a->dims[k];
  return n;
}
int mxIsDouble(const mxArray* a) { return a->kind != 1; }
int mxIsComplex(const mxArray* a) { return a->cplx; }
int mxIsEmpty(const mxArray* a) { return a->numel == 0; }
int mxIsSparse(const mxArray* a) { return a->kind == 2; }
int mxIsChar(const mxArray* a) { return a->kind == 1; }
void* mxGetData(const mxArray* a) { return a->ri ? (void*)a->ri : (void*)a->re; }
double mxGetScalar(const mxArray* a) { return a->numel ? (a->ri ? a->ri[0] : a->re[0]) : 0.0; }
int mxGetString(const mxArray* a, char* buf, mwSize n) {
  if (a->kind != 1 || strlen(a->str) + 1 > n) return 1;
  strcpy(buf, a->str);
  return 0;
}
mwIndex* mxGetJc(const mxArray* a) { return a->jc; }
mwIndex* mxGetIr(const mxArray* a) { return a->ir; }
#ifdef MX_HAS_INTERLEAVED_COMPLEX
double* mxGetDoubles(const mxArray* a) { return a->cplx ? NULL : a->re; }
mxComplexDouble* mxGetComplexDoubles(const mxArray* a) { return a->cplx ? (mxComplexDouble*)a->ri : NULL; }
#else
double* mxGetPr(const mxArray* a) { return a->re; }
double* mxGetPi(const mxArray* a) { return a->im; }
#endif

static mxArray* new_dense(mwSize ndim, const mwSize* dims, int cplx) {
  mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
  a->ndim = ndim;
  a->numel = 1;
  for (mwSize k = 0; k < ndim; ++k) {
    a->dims[k] = dims[k];
    a->numel *= dims[k];
  }
  a->cplx = cplx;
#ifdef MX_HAS_INTERLEAVED_COMPLEX
  if (cplx)
    a->ri = (double*)calloc(2 * a->numel + 1, sizeof(double));
  else
    a->re = (double*)calloc(a->numel + 1, sizeof(double));
#else
  a->re = (double*)calloc(a->numel + 1, sizeof(double));
  if (cplx) a->im = (double*)calloc(a->numel + 1, sizeof(double));
#endif
  return a;
}
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
  mwSize d[2] = {m, n};
  return new_dense(2, d, c == mxCOMPLEX);
}
mxArray* mxCreateDoubleScalar(double v) {
  mxArray* a = mxCreateDoubleMatrix(1, 1, mxREAL);
  a->re[0] = v;
  return a;
}

/* ---- test entry points ---- */
/* a dense double array from split parts (im NULL: real) */
mxArray* stub_double(int ndim, const long long* dims, const double* re, const double* im) {
  mwSize d[8];
  for (int k = 0; k < ndim; ++k) d[k] = (mwSize)dims[k];
  mxArray* a = new_dense((mwSize)ndim, d, im != NULL);
  for (size_t i = 0; i < a->numel; ++i) {
#ifdef MX_HAS_INTERLEAVED_COMPLEX
    if (im) {
      a->ri[2 * i] = re[i];
      a->ri[2 * i + 1] = im[i];
    } else {
      a->re[i] = re[i];
    }
#else
    a->re[i] = re[i];
    if (im) a->im[i] = im[i];
#endif
  }
  return a;
}
mxArray* stub_sparse(long long m, long long n, const long long* jc, const long long* ir, const double* pr) {
  mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
  a->kind = 2;
  a->ndim = 2;
  a->dims[0] = (mwSize)m;
  a->dims[1] = (mwSize)n;
  a->numel = (size_t)(m * n);
  const long long nnz = jc[n];
  a->jc = (mwIndex*)calloc((size_t)n + 1, sizeof(mwIndex));
  a->ir = (mwIndex*)calloc((size_t)nnz + 1, sizeof(mwIndex));
  a->re = (double*)calloc((size_t)nnz + 1, sizeof(double));
  for (long long j = 0; j <= n; ++j) a->jc[j] = (mwIndex)jc[j];
  for (long long k = 0; k < nnz; ++k) {
    a->ir[k] = (mwIndex)ir[k];
    a->re[k] = pr[k];
  }
  return a;
}
mxArray* stub_char(const char* s) {
  mxArray* a = (mxArray*)calloc(1, sizeof(mxArray));
  a->kind = 1;
  a->ndim = 2;
  a->dims[0] = 1;
  a->dims[1] = strlen(s);
  a->numel = strlen(s);
  a->str = (char*)malloc(strlen(s) + 1);
  strcpy(a->str, s);
  return a;
}
size_t stub_numel(const mxArray* a) { return a->numel; }
/* the array's values as split parts (im may be NULL) */
void stub_read(const mxArray* a, double* re, double* im) {
  for (size_t i = 0; i < a->numel; ++i) {
#ifdef MX_HAS_INTERLEAVED_COMPLEX
    re[i] = a->cplx ? a->ri[2 * i] : a->re[i];
    if (im) im[i] = a->cplx ? a->ri[2 * i + 1] : 0.0;
#else
    re[i] = a->re[i];
    if (im) im[i] = a->im ? a->im[i] : 0.0;
#endif
  }
}
void stub_free(mxArray* a) {
  if (!a) return;
  free(a->re);
  free(a->im);
  free(a->ri);
  free(a->jc);
  free(a->ir);
  free(a->str);
  free(a);
}
/* mexFunction with the error (identifier|text) caught: 0 on success, 1 on error */
int stub_call(int nlhs, mxArray** plhs, int nrhs, mxArray** prhs) {
  g_err[0] = 0;
  if (setjmp(g_jmp)) return 1;
  mexFunction(nlhs, plhs, nrhs, (const mxArray**)prhs);
  return 0;
}
const char* stub_error(void) { return g_err; }
int stub_interleaved(void) {
#ifdef MX_HAS_INTERLEAVED_COMPLEX
  return 1;
#else
  return 0;
#endif
}
void stub_exit(void) {
  if (g_atexit) g_atexit();
  g_atexit = NULL;
}
