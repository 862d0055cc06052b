// C ABI entry points (include/voxhenry_gpu.h): context, geometry and matvec.
#include <atomic>
#include <cstring>
#include <vector>

#include "../../include/voxhenry_gpu.h"
#include "vh_internal.cuh"

using namespace vh;

namespace vh {
static std::atomic<int64_t> g_launches{0};
int64_t launches_total() { return g_launches.load(std::memory_order_relaxed); }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int max_dyn_smem_optin() {
  static std::atomic<int> cache[64];   // per device; 0 = not looked up yet
  int dev = 0;
  VH_CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64) {
    const int v = cache[dev].load(std::memory_order_relaxed);
    if (v) return v;
  }
  int v = 0;
  VH_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (dev >= 0 && dev < 64) cache[dev].store(v, std::memory_order_relaxed);
  return v;
}
}  // namespace vh

namespace {

template <typename F>
vh_status guarded(vh_ctx* ctx, F&& f) {
  try {
    f();
    return VH_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.msg;
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return VH_ERR_OOM;
  } catch (const std::exception& e) {
    if (ctx) ctx->last_error = e.what();
    return VH_ERR_CUDA;
  }
}

__global__ void k_fill_c(double2* p, int64_t n, double2 v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// z per non-empty voxel: z_real(idxS) + z_imag(idxS)
__global__ void k_gather_z(const double* __restrict__ zr, const double2* __restrict__ zi, const int64_t* __restrict__ idx,
                           int64_t nv, double2* __restrict__ out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = idx[v] - 1;
    double2 z = make_double2(zr[li], 0.0);
    if (zi) { z.x += zi[li].x; z.y += zi[li].y; }
    out[v] = z;
  }
}

void set_z_slot(vh_geom* g, int slot, const double* z_real, const double* z_imag) {
  VH_REQUIRE(slot >= 0 && slot < 4096, ERR_BAD_ARG, "z slot out of range");
  VH_REQUIRE(z_real != nullptr, ERR_BAD_ARG, "z_real is required");
  cudaStream_t st = g->ctx->stream;
  const int64_t lmn = (int64_t)g->L * g->M * g->N;
  if ((int)g->zslots.size() <= slot) g->zslots.resize(slot + 1, nullptr);
  if (!g->zslots[slot]) VH_CUDA_TRY(cudaMalloc(&g->zslots[slot], std::max<int64_t>(1, g->nv) * sizeof(double2)));
  double* d_zr = nullptr;
  double2* d_zi = nullptr;
  int64_t* d_idx = nullptr;
  VH_CUDA_TRY(cudaMalloc(&d_zr, lmn * sizeof(double)));
  VH_CUDA_TRY(cudaMalloc(&d_idx, std::max<int64_t>(1, g->nv) * sizeof(int64_t)));
  if (z_imag) VH_CUDA_TRY(cudaMalloc(&d_zi, lmn * sizeof(double2)));
  VH_CUDA_TRY(cudaMemcpyAsync(d_zr, z_real, lmn * sizeof(double), cudaMemcpyHostToDevice, st));
  VH_CUDA_TRY(cudaMemcpyAsync(d_idx, g->idxS.data(), g->nv * sizeof(int64_t), cudaMemcpyHostToDevice, st));
  if (z_imag) VH_CUDA_TRY(cudaMemcpyAsync(d_zi, z_imag, lmn * sizeof(double2), cudaMemcpyHostToDevice, st));
  if (g->nv) {
    k_gather_z<<<256, 256, 0, st>>>(d_zr, d_zi, d_idx, g->nv, g->zslots[slot]);
    count_launch();
  }
  VH_CUDA_TRY(cudaGetLastError());
  VH_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(d_zr);
  cudaFree(d_zi);
  cudaFree(d_idx);
}

void ensure_ones(vh_geom* g, int B) {
  if (B <= g->ones_cap) return;
  cudaFree(g->ones);
  g->ones = nullptr;
  g->ones_cap = 0;
  VH_CUDA_TRY(cudaMalloc(&g->ones, B * sizeof(double2)));
  k_fill_c<<<1, 256, 0, g->ctx->stream>>>(g->ones, B, make_double2(1.0, 0.0));
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  g->ones_cap = B;
}

// Resolves per-RHS z slots to a (pointer, stride) pair.
const double2* resolve_z(vh_geom* g, int B, const int* zslot, int64_t& zstride) {
  int s0 = zslot ? zslot[0] : 0;
  bool same = true;
  for (int b = 0; zslot && b < B; ++b) same = same && zslot[b] == s0;
  auto slot_ptr = [&](int s) {
    VH_REQUIRE(s >= 0 && s < (int)g->zslots.size() && g->zslots[s], ERR_BAD_ARG, "z slot not set");
    return g->zslots[s];
  };
  if (same) {
    zstride = 0;
    return slot_ptr(s0);
  }
  const size_t need = (size_t)B * g->nv;
  if (need > g->zgather_cap) {
    cudaFree(g->zgather);
    g->zgather = nullptr;
    g->zgather_cap = 0;
    VH_CUDA_TRY(cudaMalloc(&g->zgather, need * sizeof(double2)));
    g->zgather_cap = need;
  }
  for (int b = 0; b < B; ++b)
    VH_CUDA_TRY(cudaMemcpyAsync(g->zgather + (size_t)b * g->nv, slot_ptr(zslot[b]), g->nv * sizeof(double2),
                                cudaMemcpyDeviceToDevice, g->ctx->stream));
  zstride = g->nv;
  return g->zgather;
}

}  // namespace

namespace vh {
// Full operator of lse_matvect_mult.m for B right-hand sides (device pointers, leading dimension n).
void matvec_device(vh_geom* g, int B, const double2* x, double2* y, const double2* scale, const int* zslot, Prec prec) {
  cudaStream_t st = g->ctx->stream;
  VH_REQUIRE(g->has_conv, ERR_BAD_ARG, "geometry was created without a circulant tensor");
  if (!scale) {
    ensure_ones(g, B);
    scale = g->ones;
  }
  int64_t zstride = 0;
  const double2* z = resolve_z(g, B, zslot, zstride);
  if (g->nv > 0) {
    ProfScope ps(&g->ctx->prof, prec == PREC_FP32 ? SEC_CONV32 : SEC_CONV64, st, B);
    conv_apply(g->conv, prec, B, x, g->n, y, g->n, scale, z, zstride, st);
  }
  // y_J -= Ae^T phi ; y_phi = Ae J   (lse_matvect_mult.m:138-140)
  ProfScope ps(&g->ctx->prof, SEC_INCID, st, B);
  spmv_batched(g->AeT, B, x, g->n, g->nc, y, g->n, 0, -1, st);
  spmv_batched(g->Ae, B, x, g->n, 0, y, g->n, g->nc, 0, st);
}
}  // namespace vh

extern "C" {

int vh_version(void) { return 100; }

int64_t vh_launch_count(void) { return launches_total(); }

void* vh_ctx_stream(vh_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

vh_status vh_ctx_profile(vh_ctx* ctx, int enable) {
  if (!ctx) return VH_ERR_BAD_ARG;
  return guarded(ctx, [&] {
    VH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->prof.clear();
    ctx->prof.on = enable != 0;
  });
}

vh_status vh_ctx_profile_read(vh_ctx* ctx, double* ms, int64_t* calls, int64_t* units, int nsec) {
  if (!ctx || nsec < 0) return VH_ERR_BAD_ARG;
  return guarded(ctx, [&] {
    VH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < nsec; ++i) {
      if (ms) ms[i] = 0.0;
      if (calls) calls[i] = 0;
      if (units) units[i] = 0;
    }
    for (auto& r : ctx->prof.rec) {
      if (r.sec >= nsec || !r.e1) continue;
      float t = 0.f;
      VH_CUDA_TRY(cudaEventElapsedTime(&t, r.e0, r.e1));
      if (ms) ms[r.sec] += t;
      if (calls) calls[r.sec] += 1;
      if (units) units[r.sec] += r.units;
    }
    ctx->prof.clear();
  });
}

const char* vh_status_string(vh_status s) {
  switch (s) {
    case VH_OK: return "ok";
    case VH_ERR_BAD_ARG: return "bad argument";
    case VH_ERR_OOM: return "out of device memory";
    case VH_ERR_UNSUPPORTED: return "unsupported";
    case VH_ERR_TIMEOUT: return "timeout";
    case VH_ERR_NOT_CONVERGED: return "not converged";
    case VH_ERR_CUDA: return "CUDA error";
    case VH_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

vh_status vh_ctx_create(int device, vh_ctx** out) {
  if (!out) return VH_ERR_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return VH_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return VH_ERR_BAD_ARG;
  auto* c = new vh_ctx();
  c->device = device;
  vh_status s = guarded(c, [&] {
    VH_CUDA_TRY(cudaSetDevice(device));
    VH_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  });
  if (s != VH_OK) {
    delete c;
    return s;
  }
  *out = c;
  return VH_OK;
}

void vh_ctx_destroy(vh_ctx* ctx) { vh::ctx_release(ctx); }

const char* vh_last_error(const vh_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

vh_status vh_conv_set_tuning(vh_geom* g, vh_prec prec, int y_variant, int z_variant, int max_rhs, int x_variant) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded(g->ctx, [&] {
    VH_REQUIRE(prec >= VH_PREC_FP64 && prec <= VH_PREC_DF && y_variant >= 0 && y_variant <= 3 && z_variant >= 0 &&
                   z_variant <= 3 && max_rhs >= 0 && x_variant >= 0 && x_variant <= 2,
               ERR_BAD_ARG, "bad tuning");
    VH_REQUIRE(g->has_conv, ERR_BAD_ARG, "geometry was created without a circulant tensor");
    const int Y = g->conv.Y;
    VH_REQUIRE((y_variant != 1 && y_variant != 3) || Y == 256 || Y == 512 || Y == 1024, ERR_UNSUPPORTED,
               "the register y-pass takes padded y lengths 256, 512 and 1024");
    g->conv.tune[prec] = ConvTuning{y_variant, max_rhs, x_variant, z_variant};
  });
}

vh_status vh_conv_tune(vh_geom* g, vh_prec prec, int B, int* y_variant, int* z_variant, int* max_rhs,
                       int* x_variant, double* ms_per_rhs) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded(g->ctx, [&] {
    VH_REQUIRE(prec >= VH_PREC_FP64 && prec <= VH_PREC_DF && B >= 1, ERR_BAD_ARG, "bad tuning arguments");
    VH_REQUIRE(g->has_conv && g->nv > 0, ERR_BAD_ARG, "geometry without a circulant tensor or voxels");
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    cudaStream_t st = g->ctx->stream;
    DevicePool& pool = g->ctx->pool;
    const size_t bytes = (size_t)B * g->n * sizeof(double2);
    double2* x = static_cast<double2*>(pool.get(bytes));
    double2* y = static_cast<double2*>(pool.get(bytes));
    ensure_ones(g, B);
    // the timing does not depend on the values: a constant byte pattern (finite, nonzero doubles)
    VH_CUDA_TRY(cudaMemsetAsync(x, 0x3f, bytes, st));
    ConvPlan& p = g->conv;
    const Prec pr = (Prec)prec;
    std::vector<ConvTuning> cands;
    const bool reg_ok = p.Y == 256 || p.Y == 512 || p.Y == 1024;
    const bool col_ok = p.Z <= 32;   // the one-thread-per-column z-pass takes Z = 8, 16, 32
    const bool toep_ok = pr != PREC_FP64 && ztoep_build(p, st);   // the direct z convolution (nz <= 16)
    const bool xw = pr == PREC_FP32 && xpass_warp_ok(p);   // the candidates below use the shared-memory x passes
    for (int yv : {1, 2, 3}) {
      if (yv != 2 && !reg_ok) continue;
      for (int zv : {1, 2, 3}) {
        if ((zv == 2 && !col_ok) || (zv == 3 && !toep_ok)) continue;
        cands.push_back(ConvTuning{yv, 0, xw ? 2 : 0, zv});
        for (int w : {8, 4})
          if (w < B) cands.push_back(ConvTuning{yv, w, xw ? 2 : 0, zv});
      }
    }
    cudaEvent_t e0, e1;
    VH_CUDA_TRY(cudaEventCreate(&e0));
    VH_CUDA_TRY(cudaEventCreate(&e1));
    ConvTuning best{};
    float best_ms = 0.0f;
    const ConvTuning saved = p.tune[pr];
    // the warp-per-line x passes (complex64) are timed with the best y/z choice once it is known
    try {
      for (size_t ci = 0; ci < cands.size() + (xw ? 1 : 0); ++ci) {
        ConvTuning c = ci < cands.size() ? cands[ci] : best;
        if (ci == cands.size()) c.x_variant = 1;
        p.tune[pr] = c;
        conv_apply(p, pr, B, x, g->n, y, g->n, g->ones, g->zslots[0], 0, st);   // warm-up, sizes the scratch
        float ms = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
          VH_CUDA_TRY(cudaEventRecord(e0, st));
          conv_apply(p, pr, B, x, g->n, y, g->n, g->ones, g->zslots[0], 0, st);
          VH_CUDA_TRY(cudaEventRecord(e1, st));
          VH_CUDA_TRY(cudaEventSynchronize(e1));
          float t = 0.0f;
          VH_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
          ms = std::min(ms, t);
        }
        if (best_ms == 0.0f || ms < best_ms) {
          best_ms = ms;
          best = c;
        }
      }
    } catch (...) {
      p.tune[pr] = saved;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      pool.put(x);
      pool.put(y);
      throw;
    }
    p.tune[pr] = best;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pool.put(x);
    pool.put(y);
    if (y_variant) *y_variant = best.y_variant;
    if (z_variant) *z_variant = best.z_variant;
    if (max_rhs) *max_rhs = best.max_rhs;
    if (x_variant) *x_variant = best.x_variant;
    if (ms_per_rhs) *ms_per_rhs = best_ms / B;
  });
}

vh_status vh_ctx_synchronize(vh_ctx* ctx) {
  if (!ctx) return VH_ERR_BAD_ARG;
  return guarded(ctx, [&] { VH_CUDA_TRY(cudaStreamSynchronize(ctx->stream)); });
}

vh_status vh_ctx_trim(vh_ctx* ctx) {
  if (!ctx) return VH_ERR_BAD_ARG;
  return guarded(ctx, [&] {
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    VH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));   // cached blocks may still be read by queued work
    ctx->pool.trim();
  });
}

vh_status vh_ctx_memory(vh_ctx* ctx, int64_t* in_use, int64_t* cached) {
  if (!ctx) return VH_ERR_BAD_ARG;
  size_t u = 0, c = 0;
  ctx->pool.usage(u, c);
  if (in_use) *in_use = (int64_t)u;
  if (cached) *cached = (int64_t)c;
  return VH_OK;
}

vh_status vh_geom_create(vh_ctx* ctx, int L, int M, int N, double dx, const double* fN_all, int64_t nv,
                         const int64_t* idxS, int64_t num_node, const int64_t* Ae_jc, const int64_t* Ae_ir,
                         const double* Ae_pr, const double* z_real, const double* z_imag, int want_fp32,
                         vh_geom** out) {
  if (!ctx || !out) return VH_ERR_BAD_ARG;
  *out = nullptr;
  auto* g = new vh_geom();
  g->ctx = ctx;
  ctx->refs.fetch_add(1);
  vh_status s = guarded(ctx, [&] {
    VH_REQUIRE(L >= 2 && M >= 2 && N >= 2, ERR_UNSUPPORTED, "grids thinner than 2 voxels are not supported");
    VH_REQUIRE(dx > 0 && nv >= 0 && num_node >= 0, ERR_BAD_ARG, "bad sizes");
    VH_REQUIRE(nv <= (int64_t)L * M * N, ERR_BAD_ARG, "nv exceeds the grid");
    VH_REQUIRE((nv == 0 || idxS) && Ae_jc && z_real, ERR_BAD_ARG, "null input");
    VH_REQUIRE(5 * nv < (1LL << 31), ERR_UNSUPPORTED, "too many current unknowns");
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    g->ctx = ctx;
    g->L = L; g->M = M; g->N = N; g->dx = dx;
    g->nv = nv; g->nc = 5 * nv; g->nphi = num_node; g->n = g->nc + g->nphi;
    g->idxS.assign(idxS, idxS + nv);
    cudaStream_t st = ctx->stream;
    if (fN_all) {
      const int64_t P = 8LL * L * M * N;
      double2* raw = nullptr;
      VH_CUDA_TRY(cudaMalloc(&raw, 7 * P * sizeof(double2)));
      cudaError_t e = cudaMemcpyAsync(raw, fN_all, 7 * P * sizeof(double2), cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) {
        try {
          conv_plan_create(g->conv, L, M, N, dx, raw, nv, g->idxS.data(), want_fp32 != 0, st);
        } catch (...) {
          cudaFree(raw);
          throw;
        }
      }
      cudaFree(raw);
      VH_CUDA_TRY(e);
      g->has_conv = true;
    }
    csc_upload(num_node, g->nc, Ae_jc, Ae_ir, Ae_pr, g->Ae, g->AeT, g->hAe, g->hAeT, st);
    set_z_slot(g, 0, z_real, z_imag);
  });
  if (s != VH_OK) {
    vh_geom_destroy(g);
    return s;
  }
  *out = g;
  return VH_OK;
}

vh_status vh_geom_create_generated(vh_ctx* ctx, int L, int M, int N, double dx, int64_t nv, const int64_t* idxS,
                                   int64_t num_node, const int64_t* Ae_jc, const int64_t* Ae_ir, const double* Ae_pr,
                                   const double* z_real, const double* z_imag, int want_fp32, double* st_sparse_precon,
                                   vh_geom** out) {
  if (!ctx || !out) return VH_ERR_BAD_ARG;
  *out = nullptr;
  vh_geom* g = nullptr;
  vh_status s = vh_geom_create(ctx, L, M, N, dx, nullptr, nv, idxS, num_node, Ae_jc, Ae_ir, Ae_pr, z_real, z_imag,
                               want_fp32, &g);
  if (s != VH_OK) return s;
  s = guarded(ctx, [&] {
    cudaStream_t st = ctx->stream;
    const int64_t P = 8LL * L * M * N;
    double2* fn = nullptr;
    VH_CUDA_TRY(cudaMalloc(&fn, 7 * P * sizeof(double2)));
    try {
      double2 s3[3];
      circulant_tensor_device(L, M, N, dx, fn, s3, st);
      conv_plan_create(g->conv, L, M, N, dx, fn, nv, g->idxS.data(), want_fp32 != 0, st);
      g->has_conv = true;
      if (st_sparse_precon)
        for (int i = 0; i < 3; ++i) {
          st_sparse_precon[2 * i] = s3[i].x;
          st_sparse_precon[2 * i + 1] = s3[i].y;
        }
    } catch (...) {
      cudaFree(fn);
      throw;
    }
    cudaFree(fn);
  });
  if (s != VH_OK) {
    vh_geom_destroy(g);
    return s;
  }
  *out = g;
  return VH_OK;
}

void vh_geom_destroy(vh_geom* g) { vh::geom_release(g); }

}  // extern "C"

namespace vh {
void ctx_release(vh_ctx* c) {
  if (!c || c->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

void geom_release(vh_geom* g) {
  if (!g || g->refs.fetch_sub(1) != 1) return;
  if (g->ctx) cudaSetDevice(g->ctx->device);
  conv_plan_destroy(g->conv);
  g->Ae.free_all();
  g->AeT.free_all();
  g->chol.free_all();
  cudaFree(g->pc_tmp);
  cudaFree(g->pc_phi_df);
  cudaFree(g->approx_w);
  cudaFree(g->pc_ptrs);
  for (auto* z : g->zslots) cudaFree(z);
  cudaFree(g->ones);
  cudaFree(g->io_x);
  cudaFree(g->io_y);
  cudaFree(g->io_s);
  cudaFree(g->zgather);
  vh_ctx* c = g->ctx;
  delete g;
  ctx_release(c);
}
}  // namespace vh

extern "C" {

vh_status vh_geom_sizes(const vh_geom* g, int64_t* n_curr, int64_t* n_node, int64_t* n) {
  if (!g) return VH_ERR_BAD_ARG;
  if (n_curr) *n_curr = g->nc;
  if (n_node) *n_node = g->nphi;
  if (n) *n = g->n;
  return VH_OK;
}

vh_status vh_geom_set_z(vh_geom* g, int slot, const double* z_real, const double* z_imag) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded(g->ctx, [&] {
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    set_z_slot(g, slot, z_real, z_imag);
  });
}

vh_status vh_matvec_device(vh_geom* g, int B, const void* x_dev, void* y_dev, const void* scale_dev,
                           const int* zslot, vh_prec prec) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded(g->ctx, [&] {
    VH_REQUIRE(B >= 1 && x_dev && y_dev && x_dev != y_dev, ERR_BAD_ARG, "bad matvec arguments");
    VH_REQUIRE(prec == VH_PREC_FP64 || prec == VH_PREC_FP32 || prec == VH_PREC_DF, ERR_BAD_ARG, "bad precision");
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    matvec_device(g, B, (const double2*)x_dev, (double2*)y_dev, (const double2*)scale_dev, zslot, (Prec)prec);
  });
}

vh_status vh_matvec(vh_geom* g, int B, const double* x, double* y, const double* scale, const int* zslot,
                    vh_prec prec) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded(g->ctx, [&] {
    VH_REQUIRE(B >= 1 && x && y, ERR_BAD_ARG, "bad matvec arguments");
    VH_REQUIRE(prec == VH_PREC_FP64 || prec == VH_PREC_FP32 || prec == VH_PREC_DF, ERR_BAD_ARG, "bad precision");
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    cudaStream_t st = g->ctx->stream;
    if ((size_t)B > g->io_cap) {
      cudaFree(g->io_x); cudaFree(g->io_y); cudaFree(g->io_s);
      g->io_x = g->io_y = g->io_s = nullptr;
      g->io_cap = 0;
      VH_CUDA_TRY(cudaMalloc(&g->io_x, (size_t)B * g->n * sizeof(double2)));
      VH_CUDA_TRY(cudaMalloc(&g->io_y, (size_t)B * g->n * sizeof(double2)));
      VH_CUDA_TRY(cudaMalloc(&g->io_s, (size_t)B * sizeof(double2)));
      g->io_cap = B;
    }
    const size_t bytes = (size_t)B * g->n * sizeof(double2);
    VH_CUDA_TRY(cudaMemcpyAsync(g->io_x, x, bytes, cudaMemcpyHostToDevice, st));
    const double2* sd = nullptr;
    if (scale) {
      VH_CUDA_TRY(cudaMemcpyAsync(g->io_s, scale, B * sizeof(double2), cudaMemcpyHostToDevice, st));
      sd = g->io_s;
    }
    matvec_device(g, B, g->io_x, g->io_y, sd, zslot, (Prec)prec);
    VH_CUDA_TRY(cudaMemcpyAsync(y, g->io_y, bytes, cudaMemcpyDeviceToHost, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    VH_REQUIRE(!ztoep_take_stall(st), ERR_TIMEOUT, "a z-pass gave up waiting for its staging copies");
  });
}

}  // extern "C"
