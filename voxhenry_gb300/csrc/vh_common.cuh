// Common device/host helpers for the VoxHenry GB300 library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

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

// ---------------------------------------------------------------- device memory pool
// Per-context cache of device blocks.  The solver needs large transient buffers on every call
// (the Krylov basis of a 32-RHS batch is B (m+1) n complex values, ~16 GB on a 256 x 256 x 8 grid;
// a Schur factor ~0.25 GB per frequency), and cudaMalloc / cudaFree of that size cost milliseconds
// and synchronise the device.  get() takes the smallest cached block of at least the size asked
// (and at most twice it), else allocates; put() returns a block to the cache.  An allocation that
// fails for lack of memory frees the cache and retries.  Blocks are freed when the pool is destroyed.
class DevicePool {
 public:
  void* get(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 1) + 511) & ~(size_t)511;
    std::lock_guard<std::mutex> lock(mu_);
    auto it = free_.lower_bound(bytes);
    if (it != free_.end() && it->first <= 2 * bytes) {
      void* p = it->second;
      used_[p] = it->first;
      free_.erase(it);
      return p;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
      (void)cudaGetLastError();
      trim_locked();
      e = cudaMalloc(&p, bytes);
    }
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      throw Error{e == cudaErrorMemoryAllocation ? ERR_OOM : ERR_CUDA,
                  std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    }
    used_[p] = bytes;
    return p;
  }
  void put(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(mu_);
    auto it = used_.find(p);
    if (it == used_.end()) return;
    free_.emplace(it->second, p);
    used_.erase(it);
  }
  void trim() {
    std::lock_guard<std::mutex> lock(mu_);
    trim_locked();
  }
  // bytes handed out and bytes held in the cache
  void usage(size_t& in_use, size_t& cached) {
    std::lock_guard<std::mutex> lock(mu_);
    in_use = 0;
    cached = 0;
    for (auto& kv : used_) in_use += kv.second;
    for (auto& kv : free_) cached += kv.first;
  }
  ~DevicePool() {
    trim_locked();
    for (auto& kv : used_) cudaFree(kv.first);
  }

 private:
  void trim_locked() {
    for (auto& kv : free_) cudaFree(kv.second);
    free_.clear();
  }
  std::mutex mu_;
  std::multimap<size_t, void*> free_;
  std::unordered_map<void*, size_t> used_;
};

// ---------------------------------------------------------------- dynamic shared memory
// The largest dynamic shared memory a block may opt in to on the current device.
int max_dyn_smem_optin();
// Lets `kernel` launch with `bytes` of dynamic shared memory.  The limit is a per-kernel, process-wide
// attribute shared by every host thread and context, so it is set to the device's opt-in maximum, the
// same value for every caller, and not to `bytes`: a thread launching the kernel with more than
// another thread's size then never meets a limit that thread just lowered.
template <typename K>
void allow_dyn_smem(K* kernel, size_t bytes) {
  const int mx = max_dyn_smem_optin();
  VH_REQUIRE(bytes <= (size_t)mx, ERR_UNSUPPORTED, "a kernel needs more shared memory than the device offers");
  VH_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
}

// ---------------------------------------------------------------- instrumentation
// Kernels launched by this library (every launch site calls count_launch()).
int64_t launches_total();
void count_launch();

// Named sections timed with CUDA events on the launching stream (enabled per context).
enum Section {
  SEC_CONV64 = 0,    // FFT convolution, complex128 (the five passes)
  SEC_CONV32 = 1,    // FFT convolution, complex64
  SEC_INCID = 2,     // Ae / Ae^T products of the matvec
  SEC_FACTOR = 3,    // Schur-complement factorisation
  SEC_PRECON = 4,    // preconditioner apply (incl. triangular solves)
  SEC_KRYLOV = 5,    // Gram-Schmidt, norms, combinations
  SEC_TENSOR = 6,    // circulant tensor generation
  SEC_COUNT = 7
};

struct ProfRecord {
  int sec;
  int64_t units;     // work units of the section (right-hand sides for the matvec)
  cudaEvent_t e0, e1;
};

struct Profiler {
  bool on = false;
  std::vector<ProfRecord> rec;
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
  // returns the record index, or -1 when off
  int begin(int sec, int64_t units, cudaStream_t st) {
    if (!on) return -1;
    cudaEvent_t e0 = get();
    cudaEventRecord(e0, st);
    rec.push_back({sec, units, e0, nullptr});
    return (int)rec.size() - 1;
  }
  void end(int idx, cudaStream_t st) {
    if (idx < 0 || idx >= (int)rec.size()) return;
    cudaEvent_t e1 = get();
    cudaEventRecord(e1, st);
    rec[idx].e1 = e1;
  }
  void clear() {
    for (auto& r : rec) {
      pool.push_back(r.e0);
      if (r.e1) pool.push_back(r.e1);
    }
    rec.clear();
  }
  ~Profiler() {
    clear();
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Scoped section: records begin/end events on `st` when the profiler is on.
struct ProfScope {
  Profiler* p;
  cudaStream_t st;
  int idx = -1;
  ProfScope(Profiler* prof, int sec, cudaStream_t s, int64_t units = 0) : p(prof), st(s) {
    if (p) idx = p->begin(sec, units, st);
  }
  ~ProfScope() {
    if (p) p->end(idx, st);
  }
};

}  // namespace vh
