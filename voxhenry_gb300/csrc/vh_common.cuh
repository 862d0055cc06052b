// Common device/host helpers for the VoxHenry GB300 library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

namespace vh {

// ---------------------------------------------------------------- complex types
template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };
template <typename T> using cplx = typename cplx_t<T>::type;

__host__ __device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__host__ __device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }

template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cneg(C a) { C r; r.x = -a.x; r.y = -a.y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// a * conj(b)
template <typename C> __host__ __device__ __forceinline__ C cmulc(C a, C b) {
  C r;
  r.x = a.x * b.x + a.y * b.y;
  r.y = a.y * b.x - a.x * b.y;
  return r;
}
// acc + a * b
template <typename C> __host__ __device__ __forceinline__ C cfma(C a, C b, C acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
template <typename C, typename S> __host__ __device__ __forceinline__ C cscale(C a, S s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
// multiply by -i (dir < 0) or +i (dir > 0)
template <int DIR, typename C> __host__ __device__ __forceinline__ C cmul_i(C a) {
  C r;
  if (DIR < 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
  return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }

template <typename C> __device__ __forceinline__ C czero() { C r; r.x = 0; r.y = 0; return r; }

__device__ __forceinline__ float2 to_c(double2 a, float2) { return make_float2((float)a.x, (float)a.y); }
__device__ __forceinline__ double2 to_c(double2 a, double2) { return a; }
__device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }
__device__ __forceinline__ double2 to_d(double2 a) { return a; }

// ---------------------------------------------------------------- status
enum Status {
  OK = 0,
  ERR_BAD_ARG = 1,
  ERR_OOM = 2,
  ERR_UNSUPPORTED = 3,
  ERR_TIMEOUT = 4,
  ERR_NOT_CONVERGED = 5,
  ERR_CUDA = 6,
  ERR_NO_DEVICE = 7,
};

struct Error {
  Status st;
  std::string msg;
};

#define VH_CUDA_TRY(expr)                                                                      \
  do {                                                                                         \
    cudaError_t _e = (expr);                                                                   \
    if (_e != cudaSuccess)                                                                     \
      throw ::vh::Error{_e == cudaErrorMemoryAllocation ? ::vh::ERR_OOM : ::vh::ERR_CUDA,      \
                        std::string(#expr) + ": " + cudaGetErrorString(_e)};                   \
  } while (0)

#define VH_REQUIRE(cond, status, text)                                                         \
  do {                                                                                         \
    if (!(cond)) throw ::vh::Error{status, text};                                              \
  } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace vh
