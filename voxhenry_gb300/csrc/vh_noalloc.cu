// vh_matvec_device_noalloc: the FFT matvec of vh_matvec_device without any device-memory
// allocation in the call.  It has no counterpart in the reference.
//
// Callers that cannot allocate: a host whose device memory is all handed to its own pool
// allocator (a framework's caching allocator under a memory cap), and a host whose solve loop must
// not stall -- cudaMalloc and cudaFree synchronise the whole device and so serialise the work of its
// other streams.  The regular path grows per-geometry scratch on demand (conv_plan_reserve), a unit
// scale table (ensure_ones) and a gathered z buffer for mixed slots; this path uses none of them:
//   - the FFT scratch is the fixed device array g_fft_scratch (16 MiB), the right-hand sides are
//     processed in groups that fit it, and a grid whose single right-hand side needs more is
//     rejected with VH_ERR_UNSUPPORTED;
//   - scale == NULL uses the fixed unit table g_unit_scale (64 entries, at most 64 RHS per group);
//   - right-hand sides are grouped by z slot, so no gathered z buffer is needed.
// Nothing must start at zero: every scratch element a pass reads was written by an earlier pass.
// The arrays are shared by every context on a device, so calls whose GPU work overlaps race.
// VH_PREC_DF is not taken (VH_ERR_BAD_ARG): its first product builds the pair tensor, an allocation.
// The device addresses are looked up once per device and kept for the life of the process; after a
// cudaDeviceReset (or a reset of the primary context) they are stale, so the library must not be used
// across one.
#include <cstdio>
#include <mutex>

#include "../../include/voxhenry_gpu.h"
#include "vh_internal.cuh"

using namespace vh;

namespace {

constexpr size_t kScratchBytes = VH_MATVEC_NOALLOC_SCRATCH_BYTES;
constexpr int kUnitRhs = 64;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_fft_scratch[kScratchBytes];
__device__ __align__(256) double2 g_unit_scale[kUnitRhs];

struct DeviceArrays {
  unsigned char* scratch = nullptr;
  double2* unit = nullptr;
};
std::mutex g_setup_mutex;
DeviceArrays g_arrays[kMaxDevices];

__global__ void k_fill_unit_scale(double2* p, int n) {
  const int i = threadIdx.x;
  if (i < n) p[i] = make_double2(1.0, 0.0);
}

// Device addresses of the fixed arrays on `dev` (the current device).  The first call on a device
// looks them up and fills the unit table on `st`, then waits for it.
const DeviceArrays& device_arrays(int dev, cudaStream_t st) {
  VH_REQUIRE(dev >= 0 && dev < kMaxDevices, ERR_UNSUPPORTED, "device ordinal beyond the allocation-free matvec's table");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceArrays& d = g_arrays[dev];
  if (!d.scratch) {
    void* scratch = nullptr;
    void* unit = nullptr;
    VH_CUDA_TRY(cudaGetSymbolAddress(&scratch, g_fft_scratch));
    VH_CUDA_TRY(cudaGetSymbolAddress(&unit, g_unit_scale));
    k_fill_unit_scale<<<1, kUnitRhs, 0, st>>>(static_cast<double2*>(unit), kUnitRhs);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    d.unit = static_cast<double2*>(unit);
    d.scratch = static_cast<unsigned char*>(scratch);
  }
  return d;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

void matvec_noalloc(vh_geom* g, int B, const double2* x, double2* y, const double2* scale, const int* zslot,
                    Prec prec) {
  VH_REQUIRE(g->has_conv, ERR_BAD_ARG, "geometry was created without a circulant tensor");
  cudaStream_t st = g->ctx->stream;
  auto slot_of = [&](int b) {
    const int s = zslot ? zslot[b] : 0;
    VH_REQUIRE(s >= 0 && s < (int)g->zslots.size() && g->zslots[s], ERR_BAD_ARG, "z slot not set");
    return s;
  };
  for (int b = 0; b < B; ++b) slot_of(b);
  size_t a1 = 0, b1 = 0;
  conv_scratch_bytes(g->conv, prec, a1, b1);
  const size_t per_rhs = align256(a1) + b1;
  if (g->nv > 0 && per_rhs > kScratchBytes) {
    char msg[256];
    snprintf(msg, sizeof msg,
             "the allocation-free matvec needs %zu bytes of FFT scratch per right-hand side on this grid, more than "
             "its fixed %zu bytes; use vh_matvec_device",
             per_rhs, kScratchBytes);
    throw Error{ERR_UNSUPPORTED, msg};
  }
  const DeviceArrays& d = device_arrays(g->ctx->device, st);
  if (g->nv > 0) {
    // the largest group whose scratch fits: align256(gs * a1) + gs * b1 <= kScratchBytes
    int cap = kUnitRhs;
    while (cap > 1 && align256((size_t)cap * a1) + (size_t)cap * b1 > kScratchBytes) --cap;
    int b0 = 0;
    while (b0 < B) {
      const int s = slot_of(b0);
      int e = b0 + 1;
      while (e < B && e - b0 < cap && slot_of(e) == s) ++e;
      const int gs = e - b0;
      void* sa = d.scratch;
      void* sb = d.scratch + align256((size_t)gs * a1);
      conv_apply_scratch(g->conv, prec, gs, x + (int64_t)b0 * g->n, g->n, y + (int64_t)b0 * g->n, g->n,
                         scale ? scale + b0 : d.unit, g->zslots[s], 0, sa, sb, st);
      b0 = e;
    }
  }
  // y_J -= Ae^T phi ; y_phi = Ae J   (lse_matvect_mult.m:138-140)
  spmv_batched(g->AeT, B, x, g->n, g->nc, y, g->n, 0, -1, st);
  spmv_batched(g->Ae, B, x, g->n, 0, y, g->n, g->nc, 0, st);
}

}  // namespace

extern "C" vh_status vh_matvec_device_noalloc(vh_geom* g, int B, const void* x_dev, void* y_dev,
                                              const void* scale_dev, const int* zslot, vh_prec prec) {
  if (!g) return VH_ERR_BAD_ARG;
  vh_ctx* ctx = g->ctx;
  try {
    VH_REQUIRE(B >= 1 && x_dev && y_dev && x_dev != y_dev, ERR_BAD_ARG, "bad matvec arguments");
    VH_REQUIRE(prec == VH_PREC_FP64 || prec == VH_PREC_FP32, ERR_BAD_ARG,
               "the allocation-free matvec takes VH_PREC_FP64 or VH_PREC_FP32 (VH_PREC_DF builds a pair tensor)");
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    matvec_noalloc(g, B, static_cast<const double2*>(x_dev), static_cast<double2*>(y_dev),
                   static_cast<const double2*>(scale_dev), zslot, (Prec)prec);
    return VH_OK;
  } catch (const Error& e) {
    ctx->last_error = e.msg;
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {   // host allocation (error text, z-slot checks), as every entry point
    ctx->last_error = "host allocation failed";
    return VH_ERR_OOM;
  } catch (const std::exception& e) {
    ctx->last_error = e.what();
    return VH_ERR_CUDA;
  }
}
