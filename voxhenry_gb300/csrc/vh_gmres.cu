// Batched restarted GMRES (pgmres.m / pgmres_iter.m, left preconditioner) and flexible GMRES
// (fpgmres.m / fpgmres_iter.m, right preconditioner), one Krylov space per right-hand side, plus
// the mixed-precision iterative-refinement driver (complex64 FFT matvec inside FP64 refinement).
//
// Device: matvec, preconditioner, classical Gram-Schmidt as a fused multi-dot and a fused
// update + norm, normalisation, and the basis combinations x += V y, r = V res.
// Host: per-RHS Givens rotations of the Hessenberg column (the least-squares residual of
// Hc \ rhs, pgmres_iter.m:113-121), restart bookkeeping and convergence tests.  Right-hand sides
// that converged inside a cycle drop out of the batch (the active set is compacted).
#include <cmath>
#include <complex>
#include <vector>

#include "../../include/voxhenry_gpu.h"
#include "vh_df.cuh"
#include "vh_internal.cuh"

namespace vh {
void matvec_device(vh_geom* g, int B, const double2* x, double2* y, const double2* scale, const int* zslot, Prec prec);
void precon_apply_device(vh_geom* g, int B, vh_precon* const* pcs, const double2* x, double2* y);
}  // namespace vh

using namespace vh;
using cd = std::complex<double>;

namespace {

constexpr int kChunkThreads = 256;
constexpr int kChunkElems = 4096;   // elements per reduction chunk

// partial[a][c][j] = sum_{i in chunk c} conj(V_b[j][i]) z_a[i],  j < nj,  b = act[a]
__global__ void k_multidot(const double2* __restrict__ V, int64_t ldv, int64_t ldb, const double2* __restrict__ z,
                           int64_t ldz, const int* __restrict__ act, int nj, int64_t n, double2* __restrict__ partial) {
  const int a = blockIdx.y;
  const int c = blockIdx.x;
  const int nch = gridDim.x;
  const double2* Vb = V + (int64_t)act[a] * ldb;
  const double2* za = z + (int64_t)a * ldz;
  const int64_t i0 = (int64_t)c * kChunkElems;
  const int64_t i1 = min(n, i0 + kChunkElems);
  __shared__ double2 red[kChunkThreads / 32];
  for (int j = 0; j < nj; ++j) {
    const double2* v = Vb + (int64_t)j * ldv;
    double sx = 0.0, sy = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const double2 p = v[i], q = za[i];
      sx = fma(p.x, q.x, fma(p.y, q.y, sx));
      sy = fma(p.x, q.y, fma(-p.y, q.x, sy));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(sx, sy);
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 t = make_double2(0.0, 0.0);
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t.x += red[w].x; t.y += red[w].y; }
      partial[((int64_t)a * nch + c) * nj + j] = t;
    }
    __syncthreads();
  }
}

// out[a * ldo + j] = sum_c partial[a][c][j]: one warp per j, lanes striding the chunks, then a fixed
// butterfly (deterministic order)
__global__ void k_reduce_partials(const double2* __restrict__ partial, int nch, int nj, double2* __restrict__ out,
                                  int ldo) {
  const int a = blockIdx.x;
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = threadIdx.x >> 5; j < nj; j += nw) {
    double2 t = make_double2(0.0, 0.0);
    for (int c = lane; c < nch; c += 32) {
      const double2 p = partial[((int64_t)a * nch + c) * nj + j];
      t.x += p.x;
      t.y += p.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      t.x += __shfl_xor_sync(0xffffffffu, t.x, o);
      t.y += __shfl_xor_sync(0xffffffffu, t.y, o);
    }
    if (lane == 0) out[(int64_t)a * ldo + j] = t;
  }
}

// z_a -= sum_{j<nj} h[a][j] V_b[j];  partial[a][c] = sum |z_a|^2 over the chunk
__global__ void k_cgs_update(const double2* __restrict__ V, int64_t ldv, int64_t ldb, double2* __restrict__ z,
                             int64_t ldz, const int* __restrict__ act, const double2* __restrict__ h, int ldh, int nj,
                             int64_t n, double* __restrict__ partial) {
  const int a = blockIdx.y;
  const int c = blockIdx.x;
  const int nch = gridDim.x;
  const double2* Vb = V + (int64_t)act[a] * ldb;
  double2* za = z + (int64_t)a * ldz;
  const double2* ha = h + (int64_t)a * ldh;
  const int64_t i0 = (int64_t)c * kChunkElems;
  const int64_t i1 = min(n, i0 + kChunkElems);
  double s = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    double2 q = za[i];
    for (int j = 0; j < nj; ++j) {
      const double2 v = Vb[(int64_t)j * ldv + i];
      const double2 hj = ha[j];
      q.x -= hj.x * v.x - hj.y * v.y;
      q.y -= hj.x * v.y + hj.y * v.x;
    }
    za[i] = q;
    s = fma(q.x, q.x, fma(q.y, q.y, s));
  }
  __shared__ double red[kChunkThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    partial[(int64_t)a * nch + c] = t;
  }
}

// ---- the same Gram-Schmidt steps in pair arithmetic on the FP32 pipes, for the inner GMRES of the
// mixed-precision solver.  The FP64 versions above keep GB300's FP64 pipe ~87 % busy at ~25 % of HBM
// bandwidth (4 FP64 FMAs per 16-byte basis element).  Here each FP64 operand is split into a float
// pair with integer operations (df_split) and the sums run as Dot2 accumulations (~48 bits); the
// basis and the work vectors stay complex128.
constexpr int kChunkPer = kChunkElems / kChunkThreads;   // elements per thread in a chunk

// partial[a][c][j] = sum_{i in chunk c} conj(V_b[j][i]) z_a[i], as k_multidot over chunks of
// kDotDfChunk elements: kDotDfPer per thread, their z split once and kept in registers, the V loads
// of one basis vector all issued before its arithmetic; one barrier per basis vector (the warp
// sums alternate between two shared rows)
constexpr int kDotDfPer = 4;
constexpr int kDotDfChunk = kChunkThreads * kDotDfPer;

__global__ void __launch_bounds__(kChunkThreads)
    k_multidot_df(const double2* __restrict__ V, int64_t ldv, int64_t ldb, const double2* __restrict__ z, int64_t ldz,
                  const int* __restrict__ act, int nj, int64_t n, double2* __restrict__ partial) {
  const int a = blockIdx.y;
  const int c = blockIdx.x;
  const int nch = gridDim.x;
  const double2* Vb = V + (int64_t)act[a] * ldb;
  const double2* za = z + (int64_t)a * ldz;
  const int64_t i0 = (int64_t)c * kDotDfChunk + threadIdx.x;
  dfloat zx[kDotDfPer], zy[kDotDfPer];
#pragma unroll
  for (int u = 0; u < kDotDfPer; ++u) {
    const int64_t i = i0 + (int64_t)u * kChunkThreads;
    const double2 q = i < n ? za[i] : make_double2(0.0, 0.0);
    zx[u] = df_split(q.x);
    zy[u] = df_split(q.y);
  }
  __shared__ double2 red[2][kChunkThreads / 32];
  for (int j = 0; j < nj; ++j) {
    const double2* v = Vb + (int64_t)j * ldv;
    double2 p[kDotDfPer];
#pragma unroll
    for (int u = 0; u < kDotDfPer; ++u) {
      const int64_t i = i0 + (int64_t)u * kChunkThreads;
      p[u] = i < n ? v[i] : make_double2(0.0, 0.0);
    }
    df_dot sx(dfloat(0.0f)), sy(dfloat(0.0f));
#pragma unroll
    for (int u = 0; u < kDotDfPer; ++u) {
      const dfloat px = df_split(p[u].x), py = df_split(p[u].y);
      sx.add(px, zx[u]);    // Re conj(p) q = px qx + py qy
      sx.add(py, zy[u]);
      sy.add(px, zy[u]);    // Im conj(p) q = px qy - py qx
      sy.add(-py, zx[u]);
    }
    sx.warp_sum();
    sy.warp_sum();
    if ((threadIdx.x & 31) == 0)
      red[j & 1][threadIdx.x >> 5] = make_double2(sx.value().to_double(), sy.value().to_double());
    __syncthreads();
    if (threadIdx.x == 0) {
      double2 t = make_double2(0.0, 0.0);
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t.x += red[j & 1][w].x; t.y += red[j & 1][w].y; }
      partial[((int64_t)a * nch + c) * nj + j] = t;
    }
  }
}

constexpr int kCgsDfMaxNj = 128;   // basis vectors held (split) in shared memory

// z_a -= sum_{j<nj} h[a][j] V_b[j];  partial[a][c] = sum |z_a|^2 over the chunk, as k_cgs_update
__global__ void __launch_bounds__(kChunkThreads)
    k_cgs_update_df(const double2* __restrict__ V, int64_t ldv, int64_t ldb, double2* __restrict__ z, int64_t ldz,
                    const int* __restrict__ act, const double2* __restrict__ h, int ldh, int nj, int64_t n,
                    double* __restrict__ partial) {
  const int a = blockIdx.y;
  const int c = blockIdx.x;
  const int nch = gridDim.x;
  const double2* Vb = V + (int64_t)act[a] * ldb;
  double2* za = z + (int64_t)a * ldz;
  __shared__ dfloat hs[kCgsDfMaxNj][2];
  for (int j = threadIdx.x; j < nj; j += blockDim.x) {
    const double2 hj = h[(int64_t)a * ldh + j];
    hs[j][0] = df_split(hj.x);
    hs[j][1] = df_split(hj.y);
  }
  __syncthreads();
  const int64_t i0 = (int64_t)c * kChunkElems + threadIdx.x;
  df_dot nrm(dfloat(0.0f));
  for (int u = 0; u < kChunkPer; ++u) {
    const int64_t i = i0 + (int64_t)u * kChunkThreads;
    if (i >= n) break;
    const double2 q = za[i];
    df_dot qx(df_split(q.x)), qy(df_split(q.y));
#pragma unroll 4
    for (int j = 0; j < nj; ++j) {
      const double2 v = Vb[(int64_t)j * ldv + i];
      const dfloat vx = df_split(v.x), vy = df_split(v.y);
      const dfloat hx = hs[j][0], hy = hs[j][1];
      qx.add(-hx, vx);     // Re(q - h v) = qx - hx vx + hy vy
      qx.add(hy, vy);
      qy.add(-hx, vy);     // Im(q - h v) = qy - hx vy - hy vx
      qy.add(-hy, vx);
    }
    const dfloat rx = qx.value(), ry = qy.value();
    za[i] = make_double2(rx.to_double(), ry.to_double());
    nrm.add(rx, rx);
    nrm.add(ry, ry);
  }
  double s = nrm.value().to_double();
  __shared__ double red[kChunkThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    partial[(int64_t)a * nch + c] = t;
  }
}

// norms2[a] partial sums of |x_a|^2 (x_a = x + row(a) * ldx)
__global__ void k_norm2_partial(const double2* __restrict__ x, int64_t ldx, const int* __restrict__ rows, int64_t n,
                                double* __restrict__ partial) {
  const int a = blockIdx.y;
  const int c = blockIdx.x;
  const double2* xa = x + (int64_t)(rows ? rows[a] : a) * ldx;
  const int64_t i0 = (int64_t)c * kChunkElems;
  const int64_t i1 = min(n, i0 + kChunkElems);
  double s = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 q = xa[i];
    s = fma(q.x, q.x, fma(q.y, q.y, s));
  }
  __shared__ double red[kChunkThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    partial[(int64_t)a * gridDim.x + c] = t;
  }
}

// out[a] = sqrt(sum_c partial[a][c]): one warp per RHS (launched with 32 threads), lanes striding the
// chunks, then a fixed butterfly
__global__ void k_reduce_norm(const double* __restrict__ partial, int nch, double* __restrict__ out) {
  const int a = blockIdx.x;
  double t = 0.0;
  for (int c = threadIdx.x; c < nch; c += 32) t += partial[(int64_t)a * nch + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) out[a] = sqrt(t);
}

// dst_b = src_a * (1 / nrm[a])  (zero when nrm == 0: breakdown)
__global__ void k_scale_into(const double2* __restrict__ src, int64_t lds, double2* __restrict__ dst, int64_t ldd,
                             const int* __restrict__ act, const double* __restrict__ nrm, int64_t n) {
  const int a = blockIdx.y;
  __shared__ double s_sh;   // one FP64 division per block, not per thread (GB300's FP64 pipe is slow)
  if (threadIdx.x == 0) s_sh = nrm[a] > 0.0 ? 1.0 / nrm[a] : 0.0;
  __syncthreads();
  const double s = s_sh;
  const double2* sa = src + (int64_t)a * lds;
  double2* db = dst + (int64_t)act[a] * ldd;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = sa[i];
    db[i] = make_double2(v.x * s, v.y * s);
  }
}

// dst_a = src_b  (gather rows of a batch)
__global__ void k_gather(const double2* __restrict__ src, int64_t lds, double2* __restrict__ dst, int64_t ldd,
                         const int* __restrict__ act, int64_t n) {
  const int a = blockIdx.y;
  const double2* sb = src + (int64_t)act[a] * lds;
  double2* da = dst + (int64_t)a * ldd;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    da[i] = sb[i];
}

// out_b (+)= sum_{j<cnt[a]} coef[a][j] V_b[j]   (mode 1: add, 0: assign)
__global__ void k_combine(const double2* __restrict__ V, int64_t ldv, int64_t ldb, const int* __restrict__ act,
                          const double2* __restrict__ coef, int ldc, const int* __restrict__ cnt,
                          double2* __restrict__ out, int64_t ldo, int64_t n, int mode) {
  const int a = blockIdx.y;
  const int b = act[a];
  const double2* Vb = V + (int64_t)b * ldb;
  const double2* ca = coef + (int64_t)a * ldc;
  double2* ob = out + (int64_t)b * ldo;
  const int nj = cnt[a];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = mode ? ob[i] : make_double2(0.0, 0.0);
    for (int j = 0; j < nj; ++j) {
      const double2 v = Vb[(int64_t)j * ldv + i];
      const double2 c = ca[j];
      acc.x += c.x * v.x - c.y * v.y;
      acc.y += c.x * v.y + c.y * v.x;
    }
    ob[i] = acc;
  }
}

// x_b = b_b - y_b  (residual)
__global__ void k_sub(const double2* __restrict__ bvec, const double2* __restrict__ y, double2* __restrict__ out,
                      int64_t n_total) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_total; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_double2(bvec[i].x - y[i].x, bvec[i].y - y[i].y);
}

__global__ void k_axpy_rows(double2* __restrict__ x, const double2* __restrict__ d, int64_t ld,
                            const int* __restrict__ act, int64_t n) {
  const int a = blockIdx.y;
  double2* xb = x + (int64_t)act[a] * ld;
  const double2* da = d + (int64_t)a * ld;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    xb[i].x += da[i].x;
    xb[i].y += da[i].y;
  }
}

// The context pool that solver buffers come from while a C ABI call runs on this thread (set by
// PoolScope at the call's entry); without one, DevBuf allocates and frees directly.
thread_local DevicePool* tl_pool = nullptr;
struct PoolScope {
  DevicePool* prev;
  explicit PoolScope(DevicePool* p) : prev(tl_pool) { tl_pool = p; }
  ~PoolScope() { tl_pool = prev; }
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;
  DevicePool* pool = nullptr;
  void release() {
    if (pool)
      pool->put(p);
    else
      cudaFree(p);
    p = nullptr;
    cap = 0;
    pool = nullptr;
  }
  void ensure(size_t n) {
    if (n <= cap) return;
    release();
    const size_t bytes = std::max<size_t>(1, n) * sizeof(T);
    pool = tl_pool;
    if (pool)
      p = static_cast<T*>(pool->get(bytes));
    else
      VH_CUDA_TRY(cudaMalloc(&p, bytes));
    cap = n;
  }
  ~DevBuf() { release(); }
};

unsigned grid1(int64_t n) { return (unsigned)std::min<int64_t>(4096, std::max<int64_t>(1, ceil_div(n, 256))); }

// Norms of rows (device) -> host
std::vector<double> row_norms(const double2* x, int64_t ldx, const std::vector<int>& rows, int64_t n,
                              DevBuf<int>& d_rows, DevBuf<double>& part, DevBuf<double>& out, cudaStream_t st) {
  const int na = (int)rows.size();
  std::vector<double> res(na, 0.0);
  if (na == 0) return res;
  d_rows.ensure(na);
  VH_CUDA_TRY(cudaMemcpyAsync(d_rows.p, rows.data(), na * sizeof(int), cudaMemcpyHostToDevice, st));
  const int nch = (int)std::max<int64_t>(1, ceil_div(n, kChunkElems));
  part.ensure((size_t)na * nch);
  out.ensure(na);
  k_norm2_partial<<<dim3(nch, na), kChunkThreads, 0, st>>>(x, ldx, d_rows.p, n, part.p);
  count_launch();
  k_reduce_norm<<<na, 32, 0, st>>>(part.p, nch, out.p);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  VH_CUDA_TRY(cudaMemcpyAsync(res.data(), out.p, na * sizeof(double), cudaMemcpyDeviceToHost, st));
  VH_CUDA_TRY(cudaStreamSynchronize(st));
  return res;
}

}  // namespace

namespace vh {

// Restarted (F)GMRES for B right-hand sides of the operator `op` (length op.n).  b, x: device,
// B x n (ld n).  x holds x0 on entry (zero vector allowed).  op.M empty: no preconditioner.
void gmres_core(const KrylovOps& op, int B, const double2* b, const double* tol, int m, int maxit, bool flexible,
                Prec prec, double2* x, GmresOut& out, bool true_relres, const double2* pre_Mb) {
  cudaStream_t st = op.st;
  const int64_t n = op.n;
  const bool has_M = static_cast<bool>(op.M);
  VH_REQUIRE(m >= 1 && maxit >= 1 && B >= 1, ERR_BAD_ARG, "restart and maxit must be positive");
  // ---- workspace
  DevBuf<double2> V, Zs, Xc, Wc, Zc, R, hbuf, coef, partc, d_scale;
  DevBuf<double> partr, nrm;
  DevBuf<int> d_act, d_cnt, d_rows;
  const int64_t ldv = n, ldb = (int64_t)(m + 1) * n;
  V.ensure((size_t)B * (m + 1) * n);
  if (flexible) Zs.ensure((size_t)B * m * n);
  Xc.ensure((size_t)B * n);
  Wc.ensure((size_t)B * n);
  Zc.ensure((size_t)B * n);
  R.ensure((size_t)B * n);
  hbuf.ensure((size_t)B * (m + 2));
  coef.ensure((size_t)B * (m + 2));
  d_scale.ensure(B);
  d_act.ensure(B);
  d_cnt.ensure(B);
  const int nch = (int)std::max<int64_t>(1, ceil_div(n, kChunkElems));
  const int nch_df = (int)std::max<int64_t>(1, ceil_div(n, kDotDfChunk));   // chunks of k_multidot_df
  partc.ensure((size_t)B * std::max(nch, nch_df) * (m + 1));
  partr.ensure((size_t)B * nch);
  nrm.ensure(B);
  auto apply_A = [&](const std::vector<int>& act, const double2* xin, double2* yout, Prec p) {
    op.A(act, xin, yout, p);
    out.matvecs += (int64_t)act.size();
  };
  auto apply_M = [&](const std::vector<int>& act, const double2* xin, double2* yout) {
    if (!has_M) {
      VH_CUDA_TRY(cudaMemcpyAsync(yout, xin, act.size() * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      return;
    }
    op.M(act, xin, yout);
    out.precons += (int64_t)act.size();
  };
  auto upload_act = [&](const std::vector<int>& act) {
    VH_CUDA_TRY(cudaMemcpyAsync(d_act.p, act.data(), act.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  };
  std::vector<int> all(B);
  for (int i = 0; i < B; ++i) all[i] = i;

  out.flag.assign(B, 1);
  out.inner.assign(B, 0);
  out.outer.assign(B, 0);
  out.relres.assign(B, 0.0);
  out.resvec.assign(B, {});

  // ---- initial residual r = b - A x0 (only if x0 != 0), left preconditioning of r and b
  const std::vector<double> x0n = row_norms(x, n, all, n, d_rows, partr, nrm, st);
  upload_act(all);
  bool any_x0 = false;
  for (double v : x0n) any_x0 = any_x0 || v > 0;
  if (any_x0) {
    apply_A(all, x, Wc.p, PREC_FP64);
    k_sub<<<grid1((int64_t)B * n), 256, 0, st>>>(b, Wc.p, R.p, (int64_t)B * n);
    count_launch();
  } else {
    VH_CUDA_TRY(cudaMemcpyAsync(R.p, b, (size_t)B * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  }
  std::vector<double> bnorm(B);
  if (!flexible && has_M) {
    if (pre_Mb && !any_x0) {   // M^-1 b supplied by the caller (the refinement driver already has it)
      VH_CUDA_TRY(cudaMemcpyAsync(R.p, pre_Mb, (size_t)B * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    } else {
      apply_M(all, R.p, Zc.p);
      VH_CUDA_TRY(cudaMemcpyAsync(R.p, Zc.p, (size_t)B * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    }
    if (any_x0) {
      apply_M(all, b, Zc.p);
      bnorm = row_norms(Zc.p, n, all, n, d_rows, partr, nrm, st);
    }
  } else if (any_x0) {
    bnorm = row_norms(b, n, all, n, d_rows, partr, nrm, st);
  }
  std::vector<double> rn = row_norms(R.p, n, all, n, d_rows, partr, nrm, st);
  if (!any_x0) bnorm = rn;
  std::vector<int> active;
  for (int i = 0; i < B; ++i) {
    VH_REQUIRE(bnorm[i] > 0.0, ERR_BAD_ARG, "zero right-hand side");
    out.resvec[i].push_back(rn[i] / bnorm[i]);
    if (out.resvec[i].back() > tol[i]) active.push_back(i);
  }
  // ---- restart cycles (lock-step across the batch, per-RHS early exit)
  std::vector<std::vector<cd>> H(B), Rr(B);   // unrotated / rotated Hessenberg, column-major (m+1) x m
  std::vector<std::vector<cd>> cs(B), sn(B), gv(B);
  while (!active.empty()) {
    const int na = (int)active.size();
    for (int b0 : active) {
      out.outer[b0]++;
      H[b0].assign((size_t)(m + 1) * m, cd(0));
      Rr[b0].assign((size_t)(m + 1) * m, cd(0));
      cs[b0].assign(m, cd(0));
      sn[b0].assign(m, cd(0));
      gv[b0].assign(m + 1, cd(0));
    }
    // V_0 = r / |r|
    upload_act(active);
    std::vector<double> r0 = row_norms(R.p, n, active, n, d_rows, partr, nrm, st);
    VH_CUDA_TRY(cudaMemcpyAsync(nrm.p, r0.data(), na * sizeof(double), cudaMemcpyHostToDevice, st));
    k_gather<<<dim3(grid1(n), na), 256, 0, st>>>(R.p, n, Xc.p, n, d_act.p, n);
    count_launch();
    k_scale_into<<<dim3(grid1(n), na), 256, 0, st>>>(Xc.p, n, V.p, ldb, d_act.p, nrm.p, n);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    for (int a = 0; a < na; ++a) gv[active[a]][0] = cd(r0[a], 0.0);
    std::vector<int> kdone(na, 0);           // iterations performed in this cycle
    std::vector<int> run = active;           // RHS still iterating in this cycle
    std::vector<int> pos(na);                // index of each run entry in `active`
    for (int a = 0; a < na; ++a) pos[a] = a;
    for (int k = 0; k < m && !run.empty(); ++k) {
      const int nr = (int)run.size();
      upload_act(run);
      // w = M^-1 A v_k  (left)   or   z_k = M^-1 v_k, w = A z_k  (flexible)
      k_gather<<<dim3(grid1(n), nr), 256, 0, st>>>(V.p + (int64_t)k * n, ldb, Xc.p, n, d_act.p, n);
      count_launch();
      if (flexible) {
        apply_M(run, Xc.p, Zc.p);
        upload_act(run);
        for (int a = 0; a < nr; ++a)
          VH_CUDA_TRY(cudaMemcpyAsync(Zs.p + (int64_t)run[a] * m * n + (int64_t)k * n, Zc.p + (int64_t)a * n,
                                      n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        apply_A(run, Zc.p, Wc.p, prec);
      } else {
        apply_A(run, Xc.p, Wc.p, prec);
        if (has_M) apply_M(run, Wc.p, Zc.p);
      }
      upload_act(run);
      double2* w = (flexible || !has_M) ? Wc.p : Zc.p;
      // classical Gram-Schmidt: h = V^H w ; w -= V h ; h_{k+1} = |w| (pgmres_iter.m:107-110)
      ProfScope ps(op.prof, SEC_KRYLOV, st, nr);
      // the mixed path's inner iterations take the pair-arithmetic kernels (FP32 pipes)
      const bool pair = prec == PREC_FP32 && k + 1 <= kCgsDfMaxNj;
      if (pair)
        k_multidot_df<<<dim3(nch_df, nr), kChunkThreads, 0, st>>>(V.p, ldv, ldb, w, n, d_act.p, k + 1, n, partc.p);
      else
        k_multidot<<<dim3(nch, nr), kChunkThreads, 0, st>>>(V.p, ldv, ldb, w, n, d_act.p, k + 1, n, partc.p);
      count_launch();
      k_reduce_partials<<<nr, 256, 0, st>>>(partc.p, pair ? nch_df : nch, k + 1, hbuf.p, m + 2);
      count_launch();
      if (pair)
        k_cgs_update_df<<<dim3(nch, nr), kChunkThreads, 0, st>>>(V.p, ldv, ldb, w, n, d_act.p, hbuf.p, m + 2, k + 1,
                                                                 n, partr.p);
      else
        k_cgs_update<<<dim3(nch, nr), kChunkThreads, 0, st>>>(V.p, ldv, ldb, w, n, d_act.p, hbuf.p, m + 2, k + 1, n,
                                                              partr.p);
      count_launch();
      k_reduce_norm<<<nr, 32, 0, st>>>(partr.p, nch, nrm.p);
      count_launch();
      k_scale_into<<<dim3(grid1(n), nr), 256, 0, st>>>(w, n, V.p + (int64_t)(k + 1) * n, ldb, d_act.p, nrm.p, n);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      std::vector<double2> hh((size_t)nr * (m + 2));
      std::vector<double> hn(nr);
      VH_CUDA_TRY(cudaMemcpyAsync(hh.data(), hbuf.p, hh.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaMemcpyAsync(hn.data(), nrm.p, nr * sizeof(double), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
      std::vector<int> next, next_pos;
      for (int a = 0; a < nr; ++a) {
        const int bb = run[a];
        auto& Hb = H[bb];
        auto& Rb = Rr[bb];
        for (int j = 0; j <= k; ++j) Hb[j + (size_t)k * (m + 1)] = cd(hh[(size_t)a * (m + 2) + j].x, hh[(size_t)a * (m + 2) + j].y);
        Hb[k + 1 + (size_t)k * (m + 1)] = cd(hn[a], 0.0);
        // Givens: apply previous rotations to the new column, then annihilate h_{k+1,k}
        for (int j = 0; j <= k + 1; ++j) Rb[j + (size_t)k * (m + 1)] = Hb[j + (size_t)k * (m + 1)];
        for (int j = 0; j < k; ++j) {
          const cd t1 = Rb[j + (size_t)k * (m + 1)], t2 = Rb[j + 1 + (size_t)k * (m + 1)];
          Rb[j + (size_t)k * (m + 1)] = std::conj(cs[bb][j]) * t1 + std::conj(sn[bb][j]) * t2;
          Rb[j + 1 + (size_t)k * (m + 1)] = -sn[bb][j] * t1 + cs[bb][j] * t2;
        }
        const cd p = Rb[k + (size_t)k * (m + 1)], q = Rb[k + 1 + (size_t)k * (m + 1)];
        const double den = std::sqrt(std::norm(p) + std::norm(q));
        cd c = 1.0, s = 0.0;
        if (den > 0) {
          c = p / den;
          s = q / den;
        }
        cs[bb][k] = c;
        sn[bb][k] = s;
        Rb[k + (size_t)k * (m + 1)] = std::conj(c) * p + std::conj(s) * q;
        Rb[k + 1 + (size_t)k * (m + 1)] = 0.0;
        const cd gk = gv[bb][k];
        gv[bb][k] = std::conj(c) * gk;
        gv[bb][k + 1] = -s * gk;
        const double res = std::abs(gv[bb][k + 1]);
        const int ai = pos[a];
        kdone[ai] = k + 1;
        out.resvec[bb].push_back(res / bnorm[bb]);
        const bool breakdown = !(hn[a] > 0.0);
        if (!(res < tol[bb] * bnorm[bb]) && !breakdown) {   // pgmres_iter.m:126
          next.push_back(bb);
          next_pos.push_back(ai);
        }
      }
      run.swap(next);
      pos.swap(next_pos);
    }
    // ---- cycle end: y = R^-1 g, res = rnorm e1 - H y, x += V y (or Z y), r = V res
    std::vector<double2> cy((size_t)na * (m + 2)), cr((size_t)na * (m + 2));
    std::vector<int> cnty(na), cntr(na);
    for (int a = 0; a < na; ++a) {
      const int bb = active[a];
      const int k = kdone[a];
      std::vector<cd> y(k);
      for (int i = k - 1; i >= 0; --i) {
        cd s = gv[bb][i];
        for (int j = i + 1; j < k; ++j) s -= Rr[bb][i + (size_t)j * (m + 1)] * y[j];
        y[i] = s / Rr[bb][i + (size_t)i * (m + 1)];
      }
      std::vector<cd> res(k + 1, cd(0));
      res[0] = cd(r0[a], 0.0);
      for (int j = 0; j < k; ++j)
        for (int i = 0; i <= j + 1; ++i) res[i] -= H[bb][i + (size_t)j * (m + 1)] * y[j];
      for (int j = 0; j < k; ++j) cy[(size_t)a * (m + 2) + j] = make_double2(y[j].real(), y[j].imag());
      for (int j = 0; j <= k; ++j) cr[(size_t)a * (m + 2) + j] = make_double2(res[j].real(), res[j].imag());
      cnty[a] = k;
      cntr[a] = k + 1;
      out.inner[bb] = k;
    }
    upload_act(active);
    VH_CUDA_TRY(cudaMemcpyAsync(coef.p, cy.data(), cy.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    VH_CUDA_TRY(cudaMemcpyAsync(d_cnt.p, cnty.data(), na * sizeof(int), cudaMemcpyHostToDevice, st));
    if (flexible)
      k_combine<<<dim3(grid1(n), na), 256, 0, st>>>(Zs.p, n, (int64_t)m * n, d_act.p, coef.p, m + 2, d_cnt.p, x, n, n, 1);
    else
      k_combine<<<dim3(grid1(n), na), 256, 0, st>>>(V.p, ldv, ldb, d_act.p, coef.p, m + 2, d_cnt.p, x, n, n, 1);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    // outer loop condition of pgmres.m:153: resvec(it) > tol && outit < maxit; only the RHS that
    // go on to another cycle need the restart residual r = V res
    std::vector<int> still, spos;
    for (int a = 0; a < na; ++a) {
      const int bb = active[a];
      if (out.resvec[bb].back() > tol[bb] && out.outer[bb] < maxit) {
        still.push_back(bb);
        spos.push_back(a);
      }
    }
    if (!still.empty()) {
      const int ns = (int)still.size();
      std::vector<double2> crs((size_t)ns * (m + 2));
      std::vector<int> cnts(ns);
      for (int i = 0; i < ns; ++i) {
        std::copy(cr.begin() + (size_t)spos[i] * (m + 2), cr.begin() + (size_t)(spos[i] + 1) * (m + 2),
                  crs.begin() + (size_t)i * (m + 2));
        cnts[i] = cntr[spos[i]];
      }
      upload_act(still);
      VH_CUDA_TRY(cudaMemcpyAsync(coef.p, crs.data(), crs.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
      VH_CUDA_TRY(cudaMemcpyAsync(d_cnt.p, cnts.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
      k_combine<<<dim3(grid1(n), ns), 256, 0, st>>>(V.p, ldv, ldb, d_act.p, coef.p, m + 2, d_cnt.p, R.p, n, n, 0);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    }
    active.swap(still);
  }
  // ---- true relative residual |b - A x| / |b|  (pgmres.m:181); skipped for the inner solves of
  // the refinement driver, which measures the FP64 residual itself
  if (!true_relres) {
    for (int i = 0; i < B; ++i) out.flag[i] = out.resvec[i].back() <= tol[i] ? 0 : 1;
    return;
  }
  upload_act(all);
  apply_A(all, x, Wc.p, PREC_FP64);
  k_sub<<<grid1((int64_t)B * n), 256, 0, st>>>(b, Wc.p, R.p, (int64_t)B * n);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  const std::vector<double> rr = row_norms(R.p, n, all, n, d_rows, partr, nrm, st);
  const std::vector<double> bb = row_norms(b, n, all, n, d_rows, partr, nrm, st);
  for (int i = 0; i < B; ++i) {
    out.relres[i] = rr[i] / bb[i];
    out.flag[i] = out.relres[i] <= tol[i] ? 0 : 1;
  }
}

// The VIE system of geometry g: A = the FFT matvec (scale, z slot per RHS), M = the RHS's
// preconditioners (nullptr: none).
void gmres_device(vh_geom* g, int B, vh_precon* const* pcs, const double2* b, const double2* scale_h,
                  const int* zslot_h, const double* tol, int m, int maxit, bool flexible, Prec prec, double2* x,
                  GmresOut& out, bool true_relres = true, const double2* pre_Mb = nullptr) {
  cudaStream_t st = g->ctx->stream;
  DevBuf<double2> d_scale;
  d_scale.ensure(B);
  KrylovOps op;
  op.n = g->n;
  op.st = st;
  op.prof = &g->ctx->prof;
  op.A = [&](const std::vector<int>& act, const double2* xin, double2* yout, Prec p) {
    const int na = (int)act.size();
    std::vector<double2> sc(na);
    std::vector<int> zs(na);
    for (int a = 0; a < na; ++a) {
      sc[a] = scale_h ? scale_h[act[a]] : make_double2(1.0, 0.0);
      zs[a] = zslot_h ? zslot_h[act[a]] : 0;
    }
    // a host-to-device copy from pageable memory has read its source when the call returns, so the
    // host arrays may go and the stream runs on without a host synchronisation
    VH_CUDA_TRY(cudaMemcpyAsync(d_scale.p, sc.data(), na * sizeof(double2), cudaMemcpyHostToDevice, st));
    matvec_device(g, na, xin, yout, d_scale.p, zs.data(), p);
  };
  if (pcs)
    op.M = [&](const std::vector<int>& act, const double2* xin, double2* yout) {
      std::vector<vh_precon*> ps(act.size());
      for (size_t a = 0; a < act.size(); ++a) ps[a] = pcs[act[a]];
      precon_apply_device(g, (int)act.size(), ps.data(), xin, yout);
    };
  gmres_core(op, B, b, tol, m, maxit, flexible, prec, x, out, true_relres, pre_Mb);
}

// y[a] = x[a] .* w_a (mode 0) or x[a] ./ w_a (mode 1); w_a = tab[a], a device vector of n reals
__global__ void k_rows_diag(const double2* x, double2* y, int64_t n, double* const* __restrict__ tab, int mode) {
  const int a = blockIdx.y;
  const double* w = tab[a];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = x[(int64_t)a * n + i];
    const double d = w[i];
    y[(int64_t)a * n + i] = mode ? make_double2(v.x / d, v.y / d) : make_double2(v.x * d, v.y * d);
  }
}

// phi_b = S_b^-1 bb_b approximately, S_b = Ae diag(ainv[b]) Ae^T: restarted GMRES with the Jacobi
// preconditioner diag(S_b) = sdiag[b], x0 = 0, stopping at |M^-1 r| <= tol[b] |M^-1 bb_b|
// (lse_sparse_precon_multiply.m:43: gmres(fPSchur, ., min(100, num_curr - 1), prectol, 10, precond)).
// bb: device B x nphi; phi: device, row b at phi + b * ldphi.  iters[b] = inner iterations taken.
void schur_gmres_solve(vh_geom* g, int B, double* const* ainv, double* const* sdiag, const double2* bb, double2* phi,
                       int64_t ldphi, const double* tol, int restart, int maxit, int* iters) {
  cudaStream_t st = g->ctx->stream;
  const int64_t nphi = g->nphi, nc = g->nc;
  for (int b = 0; b < B; ++b) iters[b] = 0;
  if (nphi == 0) return;
  VH_CUDA_TRY(cudaMemset2DAsync(phi, ldphi * sizeof(double2), 0, nphi * sizeof(double2), B, st));
  DevBuf<int> d_rows;
  DevBuf<double> part, nrm;
  std::vector<int> all(B);
  for (int b = 0; b < B; ++b) all[b] = b;
  const std::vector<double> nb = row_norms(bb, nphi, all, nphi, d_rows, part, nrm, st);
  std::vector<int> live;   // a zero right-hand side keeps phi = 0
  for (int b = 0; b < B; ++b)
    if (nb[b] > 0.0) live.push_back(b);
  if (live.empty()) return;
  const int nl = (int)live.size();
  DevBuf<double2> Bc, Xc, T;
  DevBuf<double*> tab;
  DevBuf<int> d_live;
  Bc.ensure((size_t)nl * nphi);
  Xc.ensure((size_t)nl * nphi);
  T.ensure((size_t)nl * std::max<int64_t>(1, nc));
  tab.ensure(nl);
  d_live.ensure(nl);
  VH_CUDA_TRY(cudaMemcpyAsync(d_live.p, live.data(), nl * sizeof(int), cudaMemcpyHostToDevice, st));
  k_gather<<<dim3(grid1(nphi), nl), 256, 0, st>>>(bb, nphi, Bc.p, nphi, d_live.p, nphi);
  count_launch();
  VH_CUDA_TRY(cudaMemsetAsync(Xc.p, 0, (size_t)nl * nphi * sizeof(double2), st));
  std::vector<double> tl(nl);
  for (int a = 0; a < nl; ++a) tl[a] = tol[live[a]];
  auto upload_tab = [&](const std::vector<int>& act, double* const* src) {
    std::vector<double*> h(act.size());
    for (size_t a = 0; a < act.size(); ++a) h[a] = src[live[act[a]]];
    VH_CUDA_TRY(cudaMemcpyAsync(tab.p, h.data(), h.size() * sizeof(double*), cudaMemcpyHostToDevice, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));   // h is consumed before it goes out of scope
  };
  KrylovOps op;
  op.n = nphi;
  op.st = st;
  op.A = [&](const std::vector<int>& act, const double2* xin, double2* yout, Prec) {   // S v = Ae (A_inv .* Ae^T v)
    const int na = (int)act.size();
    upload_tab(act, ainv);
    spmv_batched(g->AeT, na, xin, nphi, 0, T.p, nc, 0, 0, st);
    k_rows_diag<<<dim3(grid1(nc), na), 256, 0, st>>>(T.p, T.p, nc, tab.p, 0);
    count_launch();
    spmv_batched(g->Ae, na, T.p, nc, 0, yout, nphi, 0, 0, st);
    VH_CUDA_TRY(cudaGetLastError());
  };
  op.M = [&](const std::vector<int>& act, const double2* xin, double2* yout) {   // diag(S) \ v
    upload_tab(act, sdiag);
    k_rows_diag<<<dim3(grid1(nphi), (unsigned)act.size()), 256, 0, st>>>(xin, yout, nphi, tab.p, 1);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  };
  GmresOut o;
  gmres_core(op, nl, Bc.p, tl.data(), restart, maxit, false, PREC_FP64, Xc.p, o, false, nullptr);
  for (int a = 0; a < nl; ++a) {
    VH_CUDA_TRY(cudaMemcpyAsync(phi + (int64_t)live[a] * ldphi, Xc.p + (int64_t)a * nphi, nphi * sizeof(double2),
                                cudaMemcpyDeviceToDevice, st));
    iters[live[a]] = (int)o.resvec[a].size() - 1;
  }
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

// Mixed precision: iterative refinement in FP64 around complex64-matvec GMRES.
//   r = b - A x (FP64);  s = M^-1 r;  stop when |s| <= tol |M^-1 b|  (the preconditioned residual
//   that pgmres monitors);  else solve A d = r with GMRES (complex64 FFT, FP64 Krylov), x += d.
void solve_mixed_device(vh_geom* g, int B, vh_precon* const* pcs, const double2* b, const double2* scale_h,
                        const int* zslot_h, const double* tol, int m, int maxit, double inner_tol, int max_refine,
                        double2* x, GmresOut& out, std::vector<int>& refine_steps, bool has_x0) {
  cudaStream_t st = g->ctx->stream;
  const int64_t n = g->n;
  DevBuf<double2> R, S, D, Wc, Rc;
  DevBuf<double> partr, nrm;
  DevBuf<int> d_rows, d_act;
  R.ensure((size_t)B * n);
  S.ensure((size_t)B * n);
  Wc.ensure((size_t)B * n);
  std::vector<int> all(B);
  for (int i = 0; i < B; ++i) all[i] = i;
  auto Aprec = [&](const std::vector<int>& act, const double2* xin, double2* yout, Prec p) {
    const int na = (int)act.size();
    std::vector<int> zs(na);
    std::vector<double2> sc(na);
    for (int a = 0; a < na; ++a) {
      zs[a] = zslot_h ? zslot_h[act[a]] : 0;
      sc[a] = scale_h ? scale_h[act[a]] : make_double2(1.0, 0.0);
    }
    DevBuf<double2> dsc;   // pool buffers are reused in stream order
    dsc.ensure(na);
    VH_CUDA_TRY(cudaMemcpyAsync(dsc.p, sc.data(), na * sizeof(double2), cudaMemcpyHostToDevice, st));
    matvec_device(g, na, xin, yout, dsc.p, zs.data(), p);
    out.matvecs += na;
  };
  auto M = [&](const std::vector<int>& act, const double2* xin, double2* yout) {
    const int na = (int)act.size();
    if (!pcs) {
      VH_CUDA_TRY(cudaMemcpyAsync(yout, xin, (size_t)na * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      return;
    }
    std::vector<vh_precon*> ps(na);
    for (int a = 0; a < na; ++a) ps[a] = pcs[act[a]];
    precon_apply_device(g, na, ps.data(), xin, yout);
    out.precons += na;
  };
  out.flag.assign(B, 1);
  out.inner.assign(B, 0);
  out.outer.assign(B, 0);
  out.relres.assign(B, 0.0);
  out.resvec.assign(B, {});
  refine_steps.assign(B, 0);
  if (!has_x0) VH_CUDA_TRY(cudaMemsetAsync(x, 0, (size_t)B * n * sizeof(double2), st));
  // |M^-1 b|
  M(all, b, S.p);
  std::vector<double> mb = row_norms(S.p, n, all, n, d_rows, partr, nrm, st);
  const std::vector<double> bnorm = row_norms(b, n, all, n, d_rows, partr, nrm, st);
  std::vector<int> active = all;
  std::vector<double> sn = mb;      // |M^-1 r|
  std::vector<double> rn = bnorm;   // |r|
  if (has_x0) {   // r = b - A x0 (double-float product, as every refinement residual) and M^-1 r
    Aprec(all, x, Wc.p, PREC_DF);
    k_sub<<<grid1((int64_t)B * n), 256, 0, st>>>(b, Wc.p, R.p, (int64_t)B * n);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    M(all, R.p, S.p);
    sn = row_norms(S.p, n, all, n, d_rows, partr, nrm, st);
    rn = row_norms(R.p, n, all, n, d_rows, partr, nrm, st);
  } else {
    VH_CUDA_TRY(cudaMemcpyAsync(R.p, b, (size_t)B * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  }
  for (int i = 0; i < B; ++i) out.resvec[i].push_back(rn[i] / bnorm[i]);
  for (int step = 0; step < max_refine && !active.empty(); ++step) {
    const int na = (int)active.size();
    // compact r of the active RHS and solve A d = r in reduced precision
    Rc.ensure((size_t)na * n);
    D.ensure((size_t)na * n);
    d_act.ensure(na);
    VH_CUDA_TRY(cudaMemcpyAsync(d_act.p, active.data(), na * sizeof(int), cudaMemcpyHostToDevice, st));
    k_gather<<<dim3(grid1(n), na), 256, 0, st>>>(R.p, n, Rc.p, n, d_act.p, n);
    count_launch();
    VH_CUDA_TRY(cudaMemsetAsync(D.p, 0, (size_t)na * n * sizeof(double2), st));
    std::vector<double2> sc(na);
    std::vector<int> zs(na);
    std::vector<double> tl(na);
    std::vector<vh_precon*> ps(na);
    for (int a = 0; a < na; ++a) {
      const int bb = active[a];
      sc[a] = scale_h ? scale_h[bb] : make_double2(1.0, 0.0);
      zs[a] = zslot_h ? zslot_h[bb] : 0;
      // ask the inner solve for what is still missing, but not below its precision floor
      tl[a] = std::max(inner_tol, 0.5 * std::min(tol[bb] * mb[bb] / std::max(sn[bb], 1e-300),
                                                 tol[bb] * bnorm[bb] / std::max(rn[bb], 1e-300)));
      ps[a] = pcs ? pcs[bb] : nullptr;
    }
    // M^-1 r of the active rows (kept from the last check) seeds the inner solve
    DevBuf<double2> Sc;
    Sc.ensure((size_t)na * n);
    k_gather<<<dim3(grid1(n), na), 256, 0, st>>>(S.p, n, Sc.p, n, d_act.p, n);
    count_launch();
    GmresOut inner;
    gmres_device(g, na, pcs ? ps.data() : nullptr, Rc.p, sc.data(), zs.data(), tl.data(), m, maxit, false, PREC_FP32,
                 D.p, inner, false, pcs ? Sc.p : nullptr);
    out.matvecs += inner.matvecs;
    out.precons += inner.precons;
    VH_CUDA_TRY(cudaMemcpyAsync(d_act.p, active.data(), na * sizeof(int), cudaMemcpyHostToDevice, st));
    k_axpy_rows<<<dim3(grid1(n), na), 256, 0, st>>>(x, D.p, n, d_act.p, n);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    for (int a = 0; a < na; ++a) {
      const int bb = active[a];
      refine_steps[bb]++;
      out.inner[bb] += (int)inner.resvec[a].size() - 1;
      out.outer[bb] += inner.outer[a];
    }
    // New residual of the active rows, on compact copies.  After the first step it is formed in
    // FP64: r = b - A x.  After later steps it is updated, r <- r - A d, with the complex64 product
    // of the correction d: |d| ~ inner_tol |x|, so the product's relative error (~1e-6) adds about
    // 1e-11 |b| to r (classic residual updating), and an FP64 matvec per RHS and step is saved.
    std::vector<int> still;
    {
      DevBuf<double2> Ya, Sa;
      Ya.ensure((size_t)na * n);
      Sa.ensure((size_t)na * n);
      if (step == 0) {
        DevBuf<double2> Xa, Ba;
        Xa.ensure((size_t)na * n);
        Ba.ensure((size_t)na * n);
        k_gather<<<dim3(grid1(n), na), 256, 0, st>>>(x, n, Xa.p, n, d_act.p, n);
        count_launch();
        k_gather<<<dim3(grid1(n), na), 256, 0, st>>>(b, n, Ba.p, n, d_act.p, n);
        count_launch();
        Aprec(active, Xa.p, Ya.p, PREC_DF);   // ~48-bit product: far below the 1e-9.. tolerances
        k_sub<<<grid1((int64_t)na * n), 256, 0, st>>>(Ba.p, Ya.p, Ya.p, (int64_t)na * n);
        count_launch();
      } else {
        Aprec(active, D.p, Ya.p, PREC_FP32);
        k_sub<<<grid1((int64_t)na * n), 256, 0, st>>>(Rc.p, Ya.p, Ya.p, (int64_t)na * n);
        count_launch();
      }
      std::vector<int> seq(na);
      for (int a = 0; a < na; ++a) seq[a] = a;
      const std::vector<double> rnorm = row_norms(Ya.p, n, seq, n, d_rows, partr, nrm, st);
      for (int a = 0; a < na; ++a)
        VH_CUDA_TRY(cudaMemcpyAsync(R.p + (int64_t)active[a] * n, Ya.p + (int64_t)a * n, n * sizeof(double2),
                                    cudaMemcpyDeviceToDevice, st));
      // refine until the true FP64 residual meets tol: it is what the flag (pgmres.m:182-186) and the
      // accuracy of the result depend on (the preconditioner, whatever its arithmetic, sets only the
      // iteration count).  Only the RHS that go on need M^-1 r, the seed of their next inner solve.
      std::vector<int> go;   // positions in the compact arrays
      for (int a = 0; a < na; ++a) {
        const int bb = active[a];
        rn[bb] = rnorm[a];
        out.resvec[bb].push_back(rnorm[a] / bnorm[bb]);
        if (rnorm[a] > tol[bb] * bnorm[bb]) {
          go.push_back(a);
          still.push_back(bb);
        }
      }
      if (!go.empty()) {
        const int ng = (int)go.size();
        DevBuf<double2> Yg;
        DevBuf<int> d_go;
        Yg.ensure((size_t)ng * n);
        d_go.ensure(ng);
        VH_CUDA_TRY(cudaMemcpyAsync(d_go.p, go.data(), ng * sizeof(int), cudaMemcpyHostToDevice, st));
        k_gather<<<dim3(grid1(n), ng), 256, 0, st>>>(Ya.p, n, Yg.p, n, d_go.p, n);
        count_launch();
        M(still, Yg.p, Sa.p);
        std::vector<int> gseq(ng);
        for (int a = 0; a < ng; ++a) gseq[a] = a;
        const std::vector<double> snorm = row_norms(Sa.p, n, gseq, n, d_rows, partr, nrm, st);
        for (int a = 0; a < ng; ++a) {
          sn[still[a]] = snorm[a];
          VH_CUDA_TRY(cudaMemcpyAsync(S.p + (int64_t)still[a] * n, Sa.p + (int64_t)a * n, n * sizeof(double2),
                                      cudaMemcpyDeviceToDevice, st));
        }
      }
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    }
    active.swap(still);
  }
  // true relative residual: R holds b - A x (FP64) from each RHS's last refinement check
  const std::vector<double> rr = row_norms(R.p, n, all, n, d_rows, partr, nrm, st);
  const std::vector<double> bb = row_norms(b, n, all, n, d_rows, partr, nrm, st);
  for (int i = 0; i < B; ++i) {
    out.relres[i] = rr[i] / bb[i];
    out.flag[i] = out.relres[i] <= tol[i] ? 0 : 1;   // same rule as pgmres.m:182-186
  }
}

}  // namespace vh

namespace {
template <typename F>
vh_status guarded_g(vh_ctx* ctx, F&& f) {
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

namespace {
void gmres_dispatch(vh_geom* g, int B, vh_precon* const* pcs, const double2* b_dev, const double* scale,
                    const int* zslot, int restart, const double* tol, int maxit, int flexible, vh_prec prec,
                    const double2* x0_dev, double2* x_dev, int* flag, double* relres, int* iter, double* resvec,
                    int resvec_len, int* nres) {
  VH_REQUIRE(B >= 1 && b_dev && x_dev && tol, ERR_BAD_ARG, "bad gmres arguments");
  if (prec == VH_PREC_FP32 && pcs)
    for (int i = 0; i < B; ++i)
      VH_REQUIRE(pcs[i] && precon_kind(pcs[i]) != VH_PRECON_SCHUR_GMRES, ERR_UNSUPPORTED,
                 "'schur_gmres' is not a fixed operator: solve with flexible GMRES in FP64");
  VH_REQUIRE(!(flexible && prec == VH_PREC_FP32), ERR_UNSUPPORTED, "mixed precision uses the left-preconditioned form");
  PoolScope pool_scope(&g->ctx->pool);
  cudaStream_t st = g->ctx->stream;
  // x0 (pgmres.m:70): the solve starts from it; none means zero
  if (x0_dev) {
    if (x0_dev != x_dev)
      VH_CUDA_TRY(cudaMemcpyAsync(x_dev, x0_dev, (size_t)B * g->n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  } else {
    VH_CUDA_TRY(cudaMemsetAsync(x_dev, 0, (size_t)B * g->n * sizeof(double2), st));
  }
  GmresOut o;
  std::vector<int> steps;
  if (prec == VH_PREC_FP32)
    // inner tolerance 1e-5: above the complex64 floor, and two FP64 checks reach 1e-9..1e-10 (tighter
    // inner tolerances were measured to take more inner iterations in total, not fewer)
    solve_mixed_device(g, B, pcs, b_dev, (const double2*)scale, zslot, tol, restart, maxit, 1e-5, 20, x_dev, o, steps,
                       x0_dev != nullptr);
  else
    gmres_device(g, B, pcs, b_dev, (const double2*)scale, zslot, tol, restart, maxit, flexible != 0, PREC_FP64, x_dev, o);
  VH_CUDA_TRY(cudaStreamSynchronize(st));
  for (int i = 0; i < B; ++i) {
    if (flag) flag[i] = o.flag[i];
    if (relres) relres[i] = o.relres[i];
    if (iter) {
      iter[2 * i] = o.inner[i];
      iter[2 * i + 1] = o.outer[i];
    }
    if (nres) nres[i] = (int)o.resvec[i].size();
    if (resvec)
      for (int k = 0; k < resvec_len && k < (int)o.resvec[i].size(); ++k) resvec[(size_t)i * resvec_len + k] = o.resvec[i][k];
  }
}
}  // namespace

extern "C" {

vh_status vh_gmres_device_x0(vh_geom* g, int B, vh_precon* const* pcs, const void* b_dev, const double* scale,
                             const int* zslot, int restart, const double* tol, int maxit, int flexible, vh_prec prec,
                             const void* x0_dev, void* x_dev, int* flag, double* relres, int* iter, double* resvec,
                             int resvec_len, int* nres) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded_g(g->ctx, [&] {
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    gmres_dispatch(g, B, pcs, (const double2*)b_dev, scale, zslot, restart, tol, maxit, flexible, prec,
                   (const double2*)x0_dev, (double2*)x_dev, flag, relres, iter, resvec, resvec_len, nres);
    VH_REQUIRE(!ztoep_take_stall(g->ctx->stream), ERR_TIMEOUT, "a z-pass gave up waiting for its staging copies");
  });
}

vh_status vh_gmres_device(vh_geom* g, int B, vh_precon* const* pcs, const void* b_dev, const double* scale,
                          const int* zslot, int restart, const double* tol, int maxit, int flexible, vh_prec prec,
                          void* x_dev, int* flag, double* relres, int* iter, double* resvec, int resvec_len, int* nres) {
  return vh_gmres_device_x0(g, B, pcs, b_dev, scale, zslot, restart, tol, maxit, flexible, prec, nullptr, x_dev, flag,
                            relres, iter, resvec, resvec_len, nres);
}

vh_status vh_gmres_x0(vh_geom* g, int B, vh_precon* const* pcs, const double* b, const double* scale, const int* zslot,
                      int restart, const double* tol, int maxit, int flexible, vh_prec prec, const double* x0,
                      double* x, int* flag, double* relres, int* iter, double* resvec, int resvec_len, int* nres) {
  if (!g) return VH_ERR_BAD_ARG;
  return guarded_g(g->ctx, [&] {
    VH_REQUIRE(B >= 1 && b && x && tol, ERR_BAD_ARG, "bad gmres arguments");
    VH_CUDA_TRY(cudaSetDevice(g->ctx->device));
    cudaStream_t st = g->ctx->stream;
    const int64_t n = g->n;
    PoolScope pool_scope(&g->ctx->pool);   // the staging buffers come from the context pool too
    DevBuf<double2> db, dx;
    db.ensure((size_t)B * n);
    dx.ensure((size_t)B * n);
    VH_CUDA_TRY(cudaMemcpyAsync(db.p, b, (size_t)B * n * sizeof(double2), cudaMemcpyHostToDevice, st));
    if (x0) VH_CUDA_TRY(cudaMemcpyAsync(dx.p, x0, (size_t)B * n * sizeof(double2), cudaMemcpyHostToDevice, st));
    gmres_dispatch(g, B, pcs, db.p, scale, zslot, restart, tol, maxit, flexible, prec, x0 ? dx.p : nullptr, dx.p, flag,
                   relres, iter, resvec, resvec_len, nres);
    VH_CUDA_TRY(cudaMemcpyAsync(x, dx.p, (size_t)B * n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    VH_REQUIRE(!ztoep_take_stall(st), ERR_TIMEOUT, "a z-pass gave up waiting for its staging copies");
  });
}

vh_status vh_gmres(vh_geom* g, int B, vh_precon* const* pcs, const double* b, const double* scale, const int* zslot,
                   int restart, const double* tol, int maxit, int flexible, vh_prec prec, double* x, int* flag,
                   double* relres, int* iter, double* resvec, int resvec_len, int* nres) {
  return vh_gmres_x0(g, B, pcs, b, scale, zslot, restart, tol, maxit, flexible, prec, nullptr, x, flag, relres, iter,
                     resvec, resvec_len, nres);
}

}  // extern "C"
