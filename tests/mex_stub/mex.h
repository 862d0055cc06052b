/* mex.h stand-in: the subset of the MATLAB / Octave MEX API that voxhenry_gpu_mex.c uses, so that the
 * gateway builds and runs in the tests without MATLAB or Octave (mex_stub.c implements it).  Defining
 * MX_HAS_INTERLEAVED_COMPLEX gives the R2018a interleaved-complex API; without it, the split
 * real / imaginary API of earlier releases and Octave. */
#ifndef VH_MEX_STUB_H
#define VH_MEX_STUB_H
#include <stddef.h>

typedef size_t mwSize;
typedef size_t mwIndex;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;
typedef struct {
  double real, imag;
} mxComplexDouble;

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexAtExit(void (*fn)(void));
void* mxMalloc(size_t n);
void mxFree(void* p);

size_t mxGetNumberOfElements(const mxArray* a);
mwSize mxGetNumberOfDimensions(const mxArray* a);
const mwSize* mxGetDimensions(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
int mxIsDouble(const mxArray* a);
int mxIsComplex(const mxArray* a);
int mxIsEmpty(const mxArray* a);
int mxIsSparse(const mxArray* a);
int mxIsChar(const mxArray* a);
void* mxGetData(const mxArray* a);
double mxGetScalar(const mxArray* a);
int mxGetString(const mxArray* a, char* buf, mwSize n);
mwIndex* mxGetJc(const mxArray* a);
mwIndex* mxGetIr(const mxArray* a);
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray* mxCreateDoubleScalar(double v);
#ifdef MX_HAS_INTERLEAVED_COMPLEX
double* mxGetDoubles(const mxArray* a);
mxComplexDouble* mxGetComplexDoubles(const mxArray* a);
#else
double* mxGetPr(const mxArray* a);
double* mxGetPi(const mxArray* a);
#endif

#endif
