// Schur-complement block preconditioner of the [Z -Ar^T; Ar 0] system.
//
// prepare (lse_sparse_precon_prepare.m:33-64, 90-154):
//   A_inv = |1 / (z/dx + st1)| (Jx,Jy,Jz), |1 / (z/(6dx) + st2)| (J2D), |1 / (z/(2dx) + st3)| (J3D), real;
//   S = Ar A_inv Ar^T, factored (sparse Cholesky; the reference uses CHOLMOD LDL^T or LU).
// multiply (lse_sparse_precon_multiply.m:61-88):
//   bb = x_phi - Ar (A_inv x_J);  phi = S^-1 bb;  y_J = (x_J + Ar^T phi) A_inv;  y_phi = phi.
#include <cmath>
#include <vector>

#include "../../include/voxhenry_gpu.h"
#include "vh_df.cuh"
#include "vh_internal.cuh"

struct vh_precon {
  vh_geom* g = nullptr;
  int kind = 0;
  bool df = false;           // factor and triangular solves in double-float (VH_PRECON_SCHUR_INVERT_DF)
  double* A_inv = nullptr;   // nc reals
  void* W = nullptr;         // factor storage: w_total doubles, or w_total FP32 pairs when `df`;
                             // 'schur_gmres': diag(S), nphi doubles
  double prectol = 0.1;      // 'schur_gmres' inner tolerance
  int64_t inner_iters = 0;   // 'schur_gmres' inner iterations over all applies
};

namespace vh {

constexpr int kLeafPanels = 64;

__global__ void k_a_inv(const double2* __restrict__ z, int64_t nv, double dx, double2 s1, double2 s2, double2 s3,
                        double* __restrict__ out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const double2 zz = z[v];
    const double2 st[3] = {s1, s2, s3};
    const double sc[3] = {1.0 / dx, 1.0 / (6.0 * dx), 1.0 / (2.0 * dx)};
    double a[3];
    for (int k = 0; k < 3; ++k) {
      const double re = zz.x * sc[k] + st[k].x, im = zz.y * sc[k] + st[k].y;
      a[k] = 1.0 / hypot(re, im);        // |1/w| = 1/|w|
    }
    out[v] = a[0];
    out[nv + v] = a[0];
    out[2 * nv + v] = a[0];
    out[3 * nv + v] = a[1];
    out[4 * nv + v] = a[2];
  }
}

// d[r] = S(r, r) = sum_k Ae(r, k)^2 A_inv[k]  (the Jacobi preconditioner `precond` of
// lse_sparse_precon_prepare.m:85-86)
__global__ void k_schur_diag(int64_t nphi, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const double* __restrict__ val, const double* __restrict__ ainv, double* __restrict__ d) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nphi) return;
  double s = 0.0;
  for (int32_t k = rp[r]; k < rp[r + 1]; ++k) s = fma(val[k] * val[k], ainv[col[k]], s);
  d[r] = s;
}

// phi[b] = x_phi[b] - Ar (A_inv_b .* x_J[b]), stored as C: complex128 in place in y, or the
// pair-complex vector of a double-float factor; RHS b at phi + b * ldphi
template <typename C>
__global__ void k_precon_rhs(int64_t nphi, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                             const double* __restrict__ val, double* const* __restrict__ ainv,
                             const double2* __restrict__ x, int64_t ld, int64_t nc, C* __restrict__ phi,
                             int64_t ldphi) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (r >= nphi) return;
  const double2* xb = x + b * ld;
  const double* ai = ainv[b];
  double2 acc = xb[nc + r];
  for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
    const int32_t q = col[k];
    const double a = val[k] * ai[q];
    acc.x -= a * xb[q].x;
    acc.y -= a * xb[q].y;
  }
  phi[b * ldphi + r] = to_c(acc, C());
}

// the same for the double-float factor, on the FP32 pipes: the FP64 operands are split into pairs
// with integer operations (df_split) and each row's sum runs as a Dot2 accumulation, so neither the
// arithmetic nor the conversion of phi to pairs uses GB300's FP64 pipe
__global__ void k_precon_rhs_df(int64_t nphi, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                const double* __restrict__ val, double* const* __restrict__ ainv,
                                const double2* __restrict__ x, int64_t ld, int64_t nc, dcomplex* __restrict__ phi,
                                int64_t ldphi) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (r >= nphi) return;
  const double2* xb = x + b * ld;
  const double* ai = ainv[b];
  const double2 x0 = xb[nc + r];
  df_dot ax(df_split(x0.x)), ay(df_split(x0.y));
  for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
    const int32_t q = col[k];
    const dfloat a = df_split(val[k]) * df_split(ai[q]);
    const double2 xq = xb[q];
    ax.add(-a, df_split(xq.x));
    ay.add(-a, df_split(xq.y));
  }
  phi[b * ldphi + r] = dcomplex{ax.value(), ay.value()};
}

// y_J[b] = (x_J[b] + Ar^T phi[b]) .* A_inv_b;  y_phi[b] = phi[b] when phi is not y's own storage
template <typename C>
__global__ void k_precon_finish(int64_t nc, int64_t nphi, const int32_t* __restrict__ rp,
                                const int32_t* __restrict__ col, const double* __restrict__ val,
                                double* const* __restrict__ ainv, const double2* __restrict__ x,
                                double2* __restrict__ y, int64_t ld, const C* __restrict__ phi, int64_t ldphi,
                                bool copy_phi) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  const C* pb = phi + b * ldphi;
  if (q < nc) {
    double2 acc = x[b * ld + q];
    for (int32_t k = rp[q]; k < rp[q + 1]; ++k) {
      const double a = val[k];
      const double2 v = to_d(pb[col[k]]);
      acc.x = fma(a, v.x, acc.x);
      acc.y = fma(a, v.y, acc.y);
    }
    const double s = ainv[b][q];
    y[b * ld + q] = make_double2(acc.x * s, acc.y * s);
  } else if (copy_phi && q < nc + nphi) {
    y[b * ld + q] = to_d(pb[q - nc]);
  }
}

// y[b][r] = x[b][r] * w[r]  (x, y may alias)
__global__ void k_row_scale(const double2* x, int64_t ldx, const double* __restrict__ w, double2* y, int64_t ldy,
                            int64_t rows) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (r >= rows) return;
  const double2 v = x[b * ldx + r];
  y[b * ldy + r] = make_double2(v.x * w[r], v.y * w[r]);
}

// x[b][q] /= A_inv_b[q]  (the diagonal A_noninv of lse_sparse_precon_prepare.m:76)
__global__ void k_div_ainv(double2* x, int64_t ldx, double* const* __restrict__ ainv, int64_t rows) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (q >= rows) return;
  const double a = ainv[b][q];
  double2 v = x[b * ldx + q];
  v.x /= a;
  v.y /= a;
  x[b * ldx + q] = v;
}

// W = diag(1 / sum_k |Ae(r, k)|) of lse_sparse_precon_prepare.m:78, once per geometry
void ensure_approx_w(vh_geom* g) {
  if (g->approx_w || g->nphi == 0) return;
  std::vector<double> w(g->nphi);
  for (int64_t r = 0; r < g->nphi; ++r) {
    double s = 0.0;
    for (int32_t k = g->hAe.rp[r]; k < g->hAe.rp[r + 1]; ++k) s += std::fabs(g->hAe.val[k]);
    VH_REQUIRE(s > 0.0, ERR_BAD_ARG, "panel node without incident currents");
    w[r] = 1.0 / s;
  }
  VH_CUDA_TRY(cudaMalloc(&g->approx_w, g->nphi * sizeof(double)));
  VH_CUDA_TRY(cudaMemcpyAsync(g->approx_w, w.data(), g->nphi * sizeof(double), cudaMemcpyHostToDevice, g->ctx->stream));
  VH_CUDA_TRY(cudaStreamSynchronize(g->ctx->stream));
}

void ensure_symbolic(vh_geom* g) {
  if (g->chol_ready) return;
  chol_symbolic(g->chol, g->L, g->M, g->N, g->nv, g->idxS.data(), g->nphi, g->hAe.rp, g->hAe.col, g->hAe.val,
                g->hAeT.rp, g->hAeT.col, g->hAeT.val, kLeafPanels, g->ctx->stream);
  g->chol_ready = true;
}

// Applies B preconditioners (one per RHS, all of the same kind); x, y device, leading dimension n.
void precon_apply_device(vh_geom* g, int B, vh_precon* const* pcs, const double2* x, double2* y) {
  cudaStream_t st = g->ctx->stream;
  const int kind = pcs[0]->kind;
  for (int b = 0; b < B; ++b) {
    VH_REQUIRE(pcs[b] && pcs[b]->g == g, ERR_BAD_ARG, "preconditioner belongs to another geometry");
    VH_REQUIRE(pcs[b]->kind == kind, ERR_BAD_ARG, "mixed preconditioner kinds in one batch");
  }
  if (kind == VH_PRECON_NONE) {
    if (x != y) VH_CUDA_TRY(cudaMemcpyAsync(y, x, (size_t)B * g->n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    return;
  }
  VH_REQUIRE(x != y, ERR_BAD_ARG, "preconditioner apply cannot run in place");
  ProfScope ps(&g->ctx->prof, SEC_PRECON, st, B);
  if (B > g->pc_ptrs_cap) {
    cudaFree(g->pc_ptrs);
    g->pc_ptrs = nullptr;
    g->pc_ptrs_cap = 0;
    VH_CUDA_TRY(cudaMalloc(&g->pc_ptrs, 2 * (size_t)B * sizeof(double*)));
    g->pc_ptrs_cap = B;
  }
  const bool df = pcs[0]->df;
  for (int b = 0; b < B; ++b)
    VH_REQUIRE(pcs[b]->df == df, ERR_BAD_ARG, "mixed factor precisions in one batch");
  std::vector<void*> h(2 * (size_t)B);
  for (int b = 0; b < B; ++b) {
    h[b] = pcs[b]->A_inv;
    h[B + b] = pcs[b]->W;
  }
  double** d_ainv = g->pc_ptrs;
  VH_CUDA_TRY(cudaMemcpyAsync(g->pc_ptrs, h.data(), 2 * (size_t)B * sizeof(void*), cudaMemcpyHostToDevice, st));
  const size_t need = (size_t)B * std::max<int64_t>(1, g->chol.u_total);   // 16-byte complex values
  if (need > g->pc_tmp_cap) {
    cudaFree(g->pc_tmp);
    g->pc_tmp = nullptr;
    g->pc_tmp_cap = 0;
    VH_CUDA_TRY(cudaMalloc(&g->pc_tmp, need * sizeof(double2)));
    g->pc_tmp_cap = need;
  }
  if (kind == VH_PRECON_SCHUR_GMRES) {   // lse_sparse_precon_multiply.m:26-46
    const int64_t nc = g->nc, nphi = g->nphi;
    if (nphi > 0) {
      auto* bb = static_cast<double2*>(g->ctx->pool.get((size_t)B * nphi * sizeof(double2)));
      try {
        k_precon_rhs<double2><<<dim3((unsigned)ceil_div(nphi, 256), B), 256, 0, st>>>(
            nphi, g->Ae.rowptr, g->Ae.col, g->Ae.val, d_ainv, x, g->n, nc, bb, nphi);   // b - Ae A_inv a
        count_launch();
        VH_CUDA_TRY(cudaGetLastError());
        std::vector<double*> ai(B), sd(B);
        std::vector<double> tl(B);
        std::vector<int> it(B);
        for (int b = 0; b < B; ++b) {
          ai[b] = pcs[b]->A_inv;
          sd[b] = static_cast<double*>(pcs[b]->W);
          tl[b] = pcs[b]->prectol;
        }
        const int restart = (int)std::min<int64_t>(100, std::max<int64_t>(1, nc - 1));
        schur_gmres_solve(g, B, ai.data(), sd.data(), bb, y + nc, g->n, tl.data(), restart, 10, it.data());
        for (int b = 0; b < B; ++b) pcs[b]->inner_iters += it[b];
      } catch (...) {
        g->ctx->pool.put(bb);
        throw;
      }
      g->ctx->pool.put(bb);
    }
    if (nc > 0) {   // c = (a + Ae^T d) .* A_inv
      k_precon_finish<double2><<<dim3((unsigned)ceil_div(nc, 256), B), 256, 0, st>>>(
          nc, nphi, g->AeT.rowptr, g->AeT.col, g->AeT.val, d_ainv, x, y, g->n, y + nc, g->n, false);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    }
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    return;
  }
  if (kind == VH_PRECON_SCHUR_APPROX) {   // lse_sparse_precon_multiply.m:48-58
    const int64_t nc = g->nc, nphi = g->nphi;
    double2* tmp = static_cast<double2*>(g->ctx->pool.get((size_t)B * std::max<int64_t>(1, g->n) * sizeof(double2)));
    double2* t1 = tmp;                      // B x nphi
    double2* t2 = tmp + (size_t)B * nphi;   // B x nc
    if (nphi > 0) {
      const dim3 gp((unsigned)ceil_div(nphi, 256), B), gc((unsigned)std::max<int64_t>(1, ceil_div(nc, 256)), B);
      k_precon_rhs<double2><<<gp, 256, 0, st>>>(nphi, g->Ae.rowptr, g->Ae.col, g->Ae.val, d_ainv, x, g->n, nc,
                                                y + nc, g->n);   // bb
      count_launch();
      k_row_scale<<<gp, 256, 0, st>>>(y + nc, g->n, g->approx_w, t1, nphi, nphi);   // W bb
      count_launch();
      spmv_batched(g->AeT, B, t1, nphi, 0, t2, nc, 0, 0, st);                        // Ae^T W bb
      if (nc > 0) {
        k_div_ainv<<<gc, 256, 0, st>>>(t2, nc, d_ainv, nc);                          // A_noninv (...)
        count_launch();
      }
      spmv_batched(g->Ae, B, t2, nc, 0, y, g->n, nc, 0, st);                          // Ae (...)
      k_row_scale<<<gp, 256, 0, st>>>(y + nc, g->n, g->approx_w, y + nc, g->n, nphi);   // W (...)
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    }
    if (nc > 0) {
      k_precon_finish<double2><<<dim3((unsigned)ceil_div(nc, 256), B), 256, 0, st>>>(
          nc, nphi, g->AeT.rowptr, g->AeT.col, g->AeT.val, d_ainv, x, y, g->n, y + nc, g->n, false);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    }
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    g->ctx->pool.put(tmp);
    return;
  }
  dcomplex* phi_df = nullptr;
  if (df) {
    const size_t nall = (size_t)B * std::max<int64_t>(1, g->nphi);
    if (nall > g->pc_phi_df_cap) {
      cudaFree(g->pc_phi_df);
      g->pc_phi_df = nullptr;
      g->pc_phi_df_cap = 0;
      VH_CUDA_TRY(cudaMalloc(&g->pc_phi_df, nall * sizeof(dcomplex)));
      g->pc_phi_df_cap = nall;
    }
    phi_df = static_cast<dcomplex*>(g->pc_phi_df);
  }
  if (g->nphi > 0) {
    const dim3 grid((unsigned)ceil_div(g->nphi, 256), B);
    if (df) {
      k_precon_rhs_df<<<grid, 256, 0, st>>>(g->nphi, g->Ae.rowptr, g->Ae.col, g->Ae.val, d_ainv, x, g->n, g->nc,
                                            phi_df, g->nphi);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      chol_solve<dfloat>(g->chol, B, reinterpret_cast<dfloat* const*>(g->pc_ptrs + B), phi_df, g->nphi, 0,
                         reinterpret_cast<dcomplex*>(g->pc_tmp), st, y + g->nc, g->n);   // phi also into y
    } else {
      k_precon_rhs<double2><<<grid, 256, 0, st>>>(g->nphi, g->Ae.rowptr, g->Ae.col, g->Ae.val, d_ainv, x, g->n,
                                                  g->nc, y + g->nc, g->n);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      chol_solve<double>(g->chol, B, g->pc_ptrs + B, y, g->n, g->nc, g->pc_tmp, st);
    }
  }
  if (g->nc > 0) {   // phi is in y (complex128) for both factor types
    const dim3 grid((unsigned)ceil_div(g->nc, 256), B);
    k_precon_finish<double2><<<grid, 256, 0, st>>>(g->nc, g->nphi, g->AeT.rowptr, g->AeT.col, g->AeT.val, d_ainv,
                                                   x, y, g->n, y + g->nc, g->n, false);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // the pointer table was read from pageable host memory when its copy returned: no host wait here
}

int precon_kind(const vh_precon* p) { return p->kind; }

}  // namespace vh

using namespace vh;

namespace {
template <typename F>
vh_status guarded_pc(vh_ctx* ctx, F&& f) {
  try {
    f();
    return VH_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.msg;
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return VH_ERR_OOM;
  }
}
}  // namespace

extern "C" {

vh_status vh_precon_create_batch(vh_geom* g, vh_precon_kind kind, int nfreq, const double* st_sparse_precon,
                                 const int* zslot, vh_precon** out) {
  if (!g || !out || nfreq < 1) return VH_ERR_BAD_ARG;
  for (int i = 0; i < nfreq; ++i) out[i] = nullptr;
  std::vector<vh_precon*> ps(nfreq, nullptr);
  for (int i = 0; i < nfreq; ++i) {
    ps[i] = new vh_precon();
    ps[i]->g = g;
    g->refs.fetch_add(1);   // the handle keeps its geometry (and context) alive
    ps[i]->kind = kind;
  }
  vh_status s = guarded_pc(g->ctx, [&] {
    VH_REQUIRE(kind == VH_PRECON_NONE || kind == VH_PRECON_SCHUR_INVERT || kind == VH_PRECON_SCHUR_INVERT_DF ||
                   kind == VH_PRECON_SCHUR_APPROX || kind == VH_PRECON_SCHUR_GMRES,
               ERR_UNSUPPORTED, "preconditioner kind not supported (schur_invert_original)");
    const bool df = kind == VH_PRECON_SCHUR_INVERT_DF;
    const bool approx = kind == VH_PRECON_SCHUR_APPROX;
    const bool inner = kind == VH_PRECON_SCHUR_GMRES;
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    if (kind == VH_PRECON_NONE) return;
    VH_REQUIRE(st_sparse_precon, ERR_BAD_ARG, "st_sparse_precon is required");
    cudaStream_t st = g->ctx->stream;
    if (approx)
      ensure_approx_w(g);
    else if (!inner)
      ensure_symbolic(g);
    std::vector<const double*> D(nfreq);
    std::vector<void*> W(nfreq);
    for (int i = 0; i < nfreq; ++i) {
      const int zs = zslot ? zslot[i] : 0;
      VH_REQUIRE(zs >= 0 && zs < (int)g->zslots.size() && g->zslots[zs], ERR_BAD_ARG, "z slot not set");
      vh_precon* p = ps[i];
      p->A_inv = static_cast<double*>(g->ctx->pool.get(std::max<int64_t>(1, g->nc) * sizeof(double)));
      p->df = df;
      static_assert(sizeof(dfloat) == sizeof(double), "pair factor entries take a double's storage");
      if (inner)
        p->W = g->ctx->pool.get(std::max<int64_t>(1, g->nphi) * sizeof(double));
      else if (!approx)
        p->W = g->ctx->pool.get(std::max<int64_t>(1, g->chol.w_total) * sizeof(double));
      const double* sp = st_sparse_precon + 6 * i;
      const double2 s1 = make_double2(sp[0], sp[1]), s2 = make_double2(sp[2], sp[3]), s3 = make_double2(sp[4], sp[5]);
      if (g->nv) {
        k_a_inv<<<256, 256, 0, st>>>(g->zslots[zs], g->nv, g->dx, s1, s2, s3, p->A_inv);
        count_launch();
      }
      if (inner && g->nphi > 0) {
        k_schur_diag<<<(unsigned)ceil_div(g->nphi, 256), 256, 0, st>>>(g->nphi, g->Ae.rowptr, g->Ae.col, g->Ae.val,
                                                                        p->A_inv, static_cast<double*>(p->W));
        count_launch();
      }
      VH_CUDA_TRY(cudaGetLastError());
      D[i] = p->A_inv;
      W[i] = p->W;
    }
    if (approx || inner) {
      VH_CUDA_TRY(cudaStreamSynchronize(st));
      return;
    }
    ProfScope prof(&g->ctx->prof, SEC_FACTOR, st, nfreq);
    if (df)
      chol_factor<dfloat>(g->chol, nfreq, D.data(), reinterpret_cast<dfloat* const*>(W.data()), st);
    else
      chol_factor<double>(g->chol, nfreq, D.data(), reinterpret_cast<double* const*>(W.data()), st);
  });
  if (s != VH_OK) {
    for (auto* p : ps) vh_precon_destroy(p);
    return s;
  }
  for (int i = 0; i < nfreq; ++i) out[i] = ps[i];
  return VH_OK;
}

vh_status vh_precon_create(vh_geom* g, vh_precon_kind kind, const double* st_sparse_precon, int zslot,
                           vh_precon** out) {
  if (!out) return VH_ERR_BAD_ARG;
  return vh_precon_create_batch(g, kind, 1, st_sparse_precon, &zslot, out);
}

void vh_precon_destroy(vh_precon* p) {
  if (!p) return;
  vh_geom* g = p->g;
  if (g) {   // storage goes back to the context pool; the handle's reference keeps both alive until here
    cudaSetDevice(g->ctx->device);
    g->ctx->pool.put(p->A_inv);
    g->ctx->pool.put(p->W);
  }
  delete p;
  geom_release(g);
}

vh_status vh_precon_set_prectol(vh_precon* p, double prectol) {
  if (!p || !(prectol > 0.0) || !std::isfinite(prectol)) return VH_ERR_BAD_ARG;
  p->prectol = prectol;
  return VH_OK;
}

vh_status vh_precon_inner_iterations(const vh_precon* p, int64_t* total) {
  if (!p || !total) return VH_ERR_BAD_ARG;
  *total = p->inner_iters;
  return VH_OK;
}

vh_status vh_precon_stats(const vh_precon* p, int64_t* nnz_factor, double* flops, int* nfronts, int* max_front) {
  if (!p || !p->g) return VH_ERR_BAD_ARG;
  const CholSymbolic& s = p->g->chol;
  if (nnz_factor) *nnz_factor = s.nnz_l;
  if (flops) *flops = s.flops;
  if (nfronts) *nfronts = s.nfronts;
  if (max_front) *max_front = s.max_nf;
  return VH_OK;
}

vh_status vh_schur_analyze(int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t num_node,
                           const int64_t* Ae_jc, const int64_t* Ae_ir, const double* Ae_pr, int64_t* nnz_factor,
                           double* flops, int* nfronts, int* max_front, int64_t* factor_bytes) {
  try {
    VH_REQUIRE(L >= 1 && M >= 1 && N >= 1 && nv >= 0 && num_node >= 0 && Ae_jc && (nv == 0 || idxS), ERR_BAD_ARG,
               "bad arguments");
    HostCsr hA, hAT;
    csc_to_host(num_node, 5 * nv, Ae_jc, Ae_ir, Ae_pr, hA, hAT);
    CholSymbolic s;
    chol_symbolic(s, L, M, N, nv, idxS, num_node, hA.rp, hA.col, hA.val, hAT.rp, hAT.col, hAT.val, kLeafPanels,
                  nullptr, false);
    if (nnz_factor) *nnz_factor = s.nnz_l;
    if (flops) *flops = s.flops;
    if (nfronts) *nfronts = s.nfronts;
    if (max_front) *max_front = s.max_nf;
    if (factor_bytes) *factor_bytes = s.w_total * (int64_t)sizeof(double);
    return VH_OK;
  } catch (const Error& e) {
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {
    return VH_ERR_OOM;
  }
}

vh_status vh_precon_apply_device(vh_geom* g, int B, vh_precon* const* pcs, const void* x_dev, void* y_dev) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded_pc(g->ctx, [&] {
    VH_REQUIRE(B >= 1 && pcs && x_dev && y_dev, ERR_BAD_ARG, "bad preconditioner arguments");
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    precon_apply_device(g, B, pcs, (const double2*)x_dev, (double2*)y_dev);
  });
}

vh_status vh_precon_apply(vh_geom* g, int B, vh_precon* const* pcs, const double* x, double* y) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded_pc(g->ctx, [&] {
    VH_REQUIRE(B >= 1 && pcs && x && y, ERR_BAD_ARG, "bad preconditioner arguments");
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    cudaStream_t st = g->ctx->stream;
    const size_t bytes = (size_t)B * g->n * sizeof(double2);
    double2 *dx = nullptr, *dy = nullptr;
    VH_CUDA_TRY(cudaMalloc(&dx, bytes));
    cudaError_t e = cudaMalloc(&dy, bytes);
    if (e != cudaSuccess) {
      cudaFree(dx);
      VH_CUDA_TRY(e);
    }
    try {
      VH_CUDA_TRY(cudaMemcpyAsync(dx, x, bytes, cudaMemcpyHostToDevice, st));
      precon_apply_device(g, B, pcs, dx, dy);
      VH_CUDA_TRY(cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    } catch (...) {
      cudaFree(dx);
      cudaFree(dy);
      throw;
    }
    cudaFree(dx);
    cudaFree(dy);
  });
}

}  // extern "C"
