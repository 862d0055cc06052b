// Multifrontal Cholesky of S = Ar D Ar^T on the device: numeric factorisation and solves.
//
// Factor storage W: one dense nf x nf column-major block per front.  After the factorisation
// its first ns columns hold [L11; L21] and its trailing nb x nb block holds the update matrix
// passed to the parent (extend-add).  All fronts of one tree height are processed by the same
// launches; heights run from the leaves up.  Dense partial Cholesky of a front: blocks of 32
// columns -- diagonal block (one CTA), panel triangular solve (row chunks), symmetric rank-32
// update of the trailing lower triangle (64 x 64 tiles).
#include "vh_chol.cuh"

namespace vh {

constexpr int kNB = 32;   // panel width
constexpr int kTS = 64;   // update tile

// ---- assembly of the original entries of S: F(li, lj) = sum_t c_t D(q_t)
__global__ void k_chol_assemble(const FrontInfo* __restrict__ fr, const AsmEntry* __restrict__ ae,
                                const int32_t* __restrict__ aq, const double* __restrict__ ac,
                                const double* __restrict__ D, double* __restrict__ W) {
  const FrontInfo f = fr[blockIdx.x];
  double* F = W + f.w_off;
  for (int e = threadIdx.x; e < f.asm_cnt; e += blockDim.x) {
    const AsmEntry a = ae[f.asm_off + e];
    double s = 0.0;
    for (int t = a.t0; t < a.t1; ++t) s = fma(ac[t], D[aq[t]], s);
    F[a.li + (int64_t)a.lj * f.nf] = s;
  }
}

// ---- extend-add of child `which` of every front in the level list
__global__ void k_chol_extend_add(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                                  const int32_t* __restrict__ relmap, double* __restrict__ W, int which) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  const int ci = f.child[which];
  if (ci < 0) return;
  const FrontInfo c = fr[ci];
  const int nb = c.nb;
  const int32_t* rm = relmap + c.relmap_off;
  const double* U = W + c.w_off + c.ns + (int64_t)c.ns * c.nf;   // U(a, b) = U[a + b * c.nf]
  double* F = W + f.w_off;
  for (int b = blockIdx.y; b < nb; b += gridDim.y) {
    const int lj = rm[b];
    for (int a = b + threadIdx.x; a < nb; a += blockDim.x) {
      F[rm[a] + (int64_t)lj * f.nf] += U[a + (int64_t)b * c.nf];
    }
  }
}

// ---- Cholesky of the diagonal block [k0, k0+w)
__global__ void k_chol_diag(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr, double* __restrict__ W,
                            int k0, int* __restrict__ err) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  if (f.ns <= k0) return;
  const int w = min(kNB, f.ns - k0);
  __shared__ double A[kNB][kNB + 1];
  double* F = W + f.w_off;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int i = t % w, j = t / w;
    A[i][j] = (i >= j) ? F[(k0 + i) + (int64_t)(k0 + j) * f.nf] : 0.0;
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const double piv = A[j][j];
    if (!(piv > 0.0)) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      return;                                   // uniform across the CTA: piv read after a barrier
    }
    const double d = sqrt(piv);
    const double inv = 1.0 / d;
    __syncthreads();
    if (threadIdx.x == 0) A[j][j] = d;
    for (int i = j + 1 + threadIdx.x; i < w; i += blockDim.x) A[i][j] *= inv;
    __syncthreads();
    for (int t = threadIdx.x; t < (w - j - 1) * (w - j - 1); t += blockDim.x) {
      const int i = j + 1 + t % (w - j - 1), k = j + 1 + t / (w - j - 1);
      if (i >= k) A[i][k] -= A[i][j] * A[k][j];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int i = t % w, j = t / w;
    if (i >= j) F[(k0 + i) + (int64_t)(k0 + j) * f.nf] = A[i][j];
  }
}

// ---- panel rows [k0+w, nf): L(r, k0:k0+w) = F(r, k0:k0+w) L11^-T
__global__ void k_chol_panel(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr, double* __restrict__ W,
                             int k0) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  if (f.ns <= k0) return;
  const int w = min(kNB, f.ns - k0);
  const int r = k0 + w + blockIdx.y * blockDim.x + threadIdx.x;
  __shared__ double A[kNB][kNB + 1];
  double* F = W + f.w_off;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int i = t % w, j = t / w;
    A[i][j] = (i >= j) ? F[(k0 + i) + (int64_t)(k0 + j) * f.nf] : 0.0;
  }
  __syncthreads();
  if (r >= f.nf) return;
  double x[kNB];
#pragma unroll
  for (int j = 0; j < kNB; ++j)
    if (j < w) x[j] = F[r + (int64_t)(k0 + j) * f.nf];
#pragma unroll
  for (int j = 0; j < kNB; ++j) {
    if (j < w) {
      double s = x[j];
#pragma unroll
      for (int k = 0; k < kNB; ++k)
        if (k < j) s -= x[k] * A[j][k];
      x[j] = s / A[j][j];
    }
  }
#pragma unroll
  for (int j = 0; j < kNB; ++j)
    if (j < w) F[r + (int64_t)(k0 + j) * f.nf] = x[j];
}

// ---- trailing update F(r, c) -= sum_k L(r, k) L(c, k) for t0 <= c <= r < nf, k in [k0, k0+w)
__global__ void __launch_bounds__(256) k_chol_update(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                                                     double* __restrict__ W, int k0) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  if (f.ns <= k0) return;
  const int w = min(kNB, f.ns - k0);
  const int t0 = k0 + w;
  const int m = f.nf - t0;
  if (m <= 0) return;
  const int T = (m + kTS - 1) / kTS;
  const int tile = blockIdx.y;
  if (tile >= T * (T + 1) / 2) return;
  // tile -> (ti, tj), ti >= tj, row-major over the lower triangle
  int ti = (int)((sqrt(8.0 * tile + 1.0) - 1.0) * 0.5);
  while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
  while (ti * (ti + 1) / 2 > tile) --ti;
  const int tj = tile - ti * (ti + 1) / 2;
  const int r0 = t0 + ti * kTS, c0 = t0 + tj * kTS;
  __shared__ double Pr[kNB][kTS + 1];
  __shared__ double Pc[kNB][kTS + 1];
  double* F = W + f.w_off;
  for (int t = threadIdx.x; t < kNB * kTS; t += blockDim.x) {
    const int i = t % kTS, k = t / kTS;
    const int r = r0 + i, c = c0 + i;
    Pr[k][i] = (k < w && r < f.nf) ? F[r + (int64_t)(k0 + k) * f.nf] : 0.0;
    Pc[k][i] = (k < w && c < f.nf) ? F[c + (int64_t)(k0 + k) * f.nf] : 0.0;
  }
  __syncthreads();
  const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;   // 4x4 register block per thread
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int k = 0; k < w; ++k) {
    double ra[4], cb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) ra[a] = Pr[k][tr + 16 * a];
#pragma unroll
    for (int b = 0; b < 4; ++b) cb[b] = Pc[k][tc + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = fma(ra[a], cb[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int r = r0 + tr + 16 * a, c = c0 + tc + 16 * b;
      if (r < f.nf && c < f.nf && r >= c) F[r + (int64_t)c * f.nf] -= acc[a][b];
    }
}

void chol_factor(const CholSymbolic& s, const double* D, double* W, cudaStream_t st) {
  if (s.nfronts == 0) return;
  int* d_err = s.d_err;
  VH_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
  VH_CUDA_TRY(cudaMemsetAsync(W, 0, s.w_total * sizeof(double), st));
  k_chol_assemble<<<s.nfronts, 256, 0, st>>>(s.d_fronts, s.d_asm, s.d_asm_q, s.d_asm_c, D, W);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  for (size_t h = 0; h < s.levels.size(); ++h) {
    const unsigned nf = (unsigned)s.levels[h].size();
    const int32_t* lev = s.d_levels[h];
    if (h > 0) {
      const unsigned cy = (unsigned)std::min(1024, std::max(1, s.level_max_nf[h]));
      for (int which = 0; which < 2; ++which) {
        k_chol_extend_add<<<dim3(nf, cy), 128, 0, st>>>(lev, s.d_fronts, s.d_relmap, W, which);
        count_launch();
        VH_CUDA_TRY(cudaGetLastError());
      }
    }
    const int max_ns = s.level_max_ns[h];
    const int max_nf = s.level_max_nf[h];
    for (int k0 = 0; k0 < max_ns; k0 += kNB) {
      k_chol_diag<<<nf, 256, 0, st>>>(lev, s.d_fronts, W, k0, d_err);
      count_launch();
      const int rows = max_nf - k0;
      if (rows > 0) {
        k_chol_panel<<<dim3(nf, (unsigned)ceil_div(rows, 128)), 128, 0, st>>>(lev, s.d_fronts, W, k0);
        count_launch();
        const int m = max_nf - k0;
        const int T = (int)ceil_div(m, kTS);
        k_chol_update<<<dim3(nf, (unsigned)(T * (T + 1) / 2)), 256, 0, st>>>(lev, s.d_fronts, W, k0);
        count_launch();
      }
      VH_CUDA_TRY(cudaGetLastError());
    }
  }
  int herr = 0;
  VH_CUDA_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  VH_CUDA_TRY(cudaStreamSynchronize(st));
  VH_REQUIRE(herr == 0, ERR_BAD_ARG, "Schur complement is not positive definite (check the port/ground nodes)");
}

// ---- forward solve: L y = b, leaves first.  One CTA per (front, RHS).
__global__ void k_chol_fsolve(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                              const int32_t* __restrict__ rows, const int32_t* __restrict__ relmap,
                              double* const* __restrict__ Wp, double2* __restrict__ x, int64_t ldx, int64_t xoff,
                              double2* __restrict__ U, int64_t u_total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* t = reinterpret_cast<double2*>(smem_raw);
  const FrontInfo f = fr[lev[blockIdx.x]];
  const int b = blockIdx.y;
  const double* F = Wp[b] + f.w_off;
  double2* xb = x + b * ldx + xoff;
  double2* Ub = U + b * u_total;
  const int32_t* rw = rows + f.rows_off;
  for (int r = threadIdx.x; r < f.nf; r += blockDim.x) t[r] = (r < f.ns) ? xb[rw[r]] : make_double2(0.0, 0.0);
  __syncthreads();
  for (int c = 0; c < 2; ++c) {
    if (f.child[c] < 0) continue;
    const FrontInfo ch = fr[f.child[c]];
    const int32_t* rm = relmap + ch.relmap_off;
    for (int a = threadIdx.x; a < ch.nb; a += blockDim.x) {
      const double2 u = Ub[ch.u_off + a];
      double2& d = t[rm[a]];
      d.x -= u.x;
      d.y -= u.y;
    }
    __syncthreads();
  }
  for (int j = 0; j < f.ns; ++j) {
    const double inv = 1.0 / F[j + (int64_t)j * f.nf];
    const double2 y = make_double2(t[j].x * inv, t[j].y * inv);
    const double* col = F + (int64_t)j * f.nf;
    for (int r = j + 1 + threadIdx.x; r < f.nf; r += blockDim.x) {
      const double l = col[r];
      t[r].x -= l * y.x;
      t[r].y -= l * y.y;
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j < f.ns; j += blockDim.x) {
    const double inv = 1.0 / F[j + (int64_t)j * f.nf];
    xb[rw[j]] = make_double2(t[j].x * inv, t[j].y * inv);
  }
  for (int a = threadIdx.x; a < f.nb; a += blockDim.x) {
    const double2 v = t[f.ns + a];
    Ub[f.u_off + a] = make_double2(-v.x, -v.y);
  }
}

// ---- backward solve: L^T x = y, root first.
__global__ void k_chol_bsolve(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                              const int32_t* __restrict__ rows, double* const* __restrict__ Wp,
                              double2* __restrict__ x, int64_t ldx, int64_t xoff) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* t = reinterpret_cast<double2*>(smem_raw);   // nf: [z_own ; x_boundary]
  const FrontInfo f = fr[lev[blockIdx.x]];
  const int b = blockIdx.y;
  const double* F = Wp[b] + f.w_off;
  double2* xb = x + b * ldx + xoff;
  const int32_t* rw = rows + f.rows_off;
  for (int r = threadIdx.x; r < f.nf; r += blockDim.x) t[r] = xb[rw[r]];
  __syncthreads();
  // z_j -= sum_a L(ns + a, j) x_a   (one warp per column)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = warp; j < f.ns; j += nw) {
    const double* col = F + (int64_t)j * f.nf + f.ns;
    double sx = 0.0, sy = 0.0;
    for (int a = lane; a < f.nb; a += 32) {
      const double l = col[a];
      sx = fma(l, t[f.ns + a].x, sx);
      sy = fma(l, t[f.ns + a].y, sy);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (lane == 0) {
      t[j].x -= sx;
      t[j].y -= sy;
    }
  }
  __syncthreads();
  for (int j = f.ns - 1; j >= 0; --j) {
    const double inv = 1.0 / F[j + (int64_t)j * f.nf];
    const double2 xj = make_double2(t[j].x * inv, t[j].y * inv);
    for (int k = threadIdx.x; k < j; k += blockDim.x) {
      const double l = F[j + (int64_t)k * f.nf];
      t[k].x -= l * xj.x;
      t[k].y -= l * xj.y;
    }
    __syncthreads();
    if (threadIdx.x == 0) t[j] = xj;
    __syncthreads();
  }
  for (int j = threadIdx.x; j < f.ns; j += blockDim.x) xb[rw[j]] = t[j];
}

void chol_solve(const CholSymbolic& s, int B, double* const* Wp, double2* x, int64_t ldx, int64_t xoff, double2* U,
                cudaStream_t st) {
  if (s.nfronts == 0 || B == 0) return;
  const size_t sm = (size_t)s.max_nf * sizeof(double2);
  VH_REQUIRE(sm <= 200 * 1024, ERR_UNSUPPORTED, "front too large for the shared-memory solve");
  VH_CUDA_TRY(cudaFuncSetAttribute(k_chol_fsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  VH_CUDA_TRY(cudaFuncSetAttribute(k_chol_bsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  for (size_t h = 0; h < s.levels.size(); ++h) {
    const size_t smh = (size_t)s.level_max_nf[h] * sizeof(double2);
    k_chol_fsolve<<<dim3((unsigned)s.levels[h].size(), B), 256, smh, st>>>(s.d_levels[h], s.d_fronts, s.d_rows,
                                                                            s.d_relmap, Wp, x, ldx, xoff, U, s.u_total);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  for (size_t hh = s.levels.size(); hh-- > 0;) {
    const size_t smh = (size_t)s.level_max_nf[hh] * sizeof(double2);
    k_chol_bsolve<<<dim3((unsigned)s.levels[hh].size(), B), 256, smh, st>>>(s.d_levels[hh], s.d_fronts, s.d_rows, Wp,
                                                                             x, ldx, xoff);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
}

}  // namespace vh
