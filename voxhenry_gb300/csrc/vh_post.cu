// Post-processing of the solution currents on the device (src_post_process of the reference):
// the current coefficients scattered onto the voxel grid (post_obtain_curr_coefs_on_grid.m) and
// a batched real-sparse x complex product, which gives the currents on the nodes
// -Ae_only_leaving x + Ae_only_entering_bndry x of post_obtain_currs_on_nodes.m:7-9.
#include <vector>

#include "../../include/voxhenry_gpu.h"
#include "vh_internal.cuh"

using namespace vh;

namespace {

// grid[b][c][li] = x[b][c * nv + v] for the voxel v at 0-based linear index li = idxS[v] - 1
__global__ void k_scatter_currents(const double2* __restrict__ x, int64_t ldx, const int64_t* __restrict__ idxS,
                                   int64_t nv, double2* __restrict__ grid, int64_t lmn) {
  const int b = blockIdx.z, c = blockIdx.y;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x)
    grid[((int64_t)b * 5 + c) * lmn + idxS[v] - 1] = x[(int64_t)b * ldx + c * nv + v];
}

template <typename F>
vh_status guarded_post(vh_ctx* ctx, F&& f) {
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

vh_status vh_currents_on_grid(vh_ctx* ctx, int L, int M, int N, int64_t nv, const int64_t* idxS, int B,
                              const double* x, int64_t ldx, double* grids) {
  if (!ctx) return VH_ERR_BAD_ARG;
  return guarded_post(ctx, [&] {
    const int64_t lmn = (int64_t)L * M * N;
    VH_REQUIRE(L >= 1 && M >= 1 && N >= 1 && nv >= 0 && nv <= lmn && B >= 1 && ldx >= 5 * nv && x && grids &&
                   (nv == 0 || idxS),
               ERR_BAD_ARG, "bad arguments");
    for (int64_t v = 0; v < nv; ++v)
      VH_REQUIRE(idxS[v] >= 1 && idxS[v] <= lmn && (v == 0 || idxS[v] > idxS[v - 1]), ERR_BAD_ARG,
                 "idxS must be strictly increasing 1-based indices into the grid");
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    DevicePool& pool = ctx->pool;
    const size_t gbytes = (size_t)B * 5 * lmn * sizeof(double2);
    auto* d_grid = static_cast<double2*>(pool.get(gbytes));
    auto* d_x = static_cast<double2*>(pool.get((size_t)B * std::max<int64_t>(1, 5 * nv) * sizeof(double2)));
    auto* d_idx = static_cast<int64_t*>(pool.get(std::max<int64_t>(1, nv) * sizeof(int64_t)));
    try {
      VH_CUDA_TRY(cudaMemsetAsync(d_grid, 0, gbytes, st));
      if (nv > 0) {
        VH_CUDA_TRY(cudaMemcpy2DAsync(d_x, 5 * nv * sizeof(double2), x, ldx * sizeof(double2),
                                      5 * nv * sizeof(double2), B, cudaMemcpyHostToDevice, st));
        VH_CUDA_TRY(cudaMemcpyAsync(d_idx, idxS, nv * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        const dim3 grid((unsigned)std::min<int64_t>(1024, ceil_div(nv, 256)), 5, (unsigned)B);
        k_scatter_currents<<<grid, 256, 0, st>>>(d_x, 5 * nv, d_idx, nv, d_grid, lmn);
        count_launch();
        VH_CUDA_TRY(cudaGetLastError());
      }
      VH_CUDA_TRY(cudaMemcpyAsync(grids, d_grid, gbytes, cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    } catch (...) {
      pool.put(d_grid);
      pool.put(d_x);
      pool.put(d_idx);
      throw;
    }
    pool.put(d_grid);
    pool.put(d_x);
    pool.put(d_idx);
  });
}

vh_status vh_sparse_matvec(vh_ctx* ctx, int64_t nrows, int64_t ncols, const int64_t* jc, const int64_t* ir,
                           const double* pr, int B, const double* x, int64_t ldx, double* y, int64_t ldy) {
  if (!ctx) return VH_ERR_BAD_ARG;
  return guarded_post(ctx, [&] {
    VH_REQUIRE(nrows >= 0 && ncols >= 0 && B >= 1 && jc && x && y && ldx >= ncols && ldy >= nrows, ERR_BAD_ARG,
               "bad arguments");
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    HostCsr hA, hAT;   // CSR of the CSC input (hAT unused here)
    csc_to_host(nrows, ncols, jc, ir, pr, hA, hAT);
    Csr A;
    try {
      A.nrows = nrows;
      A.ncols = ncols;
      A.nnz = (int64_t)hA.col.size();
      VH_CUDA_TRY(cudaMalloc(&A.rowptr, (nrows + 1) * sizeof(int32_t)));
      VH_CUDA_TRY(cudaMalloc(&A.col, std::max<int64_t>(1, A.nnz) * sizeof(int32_t)));
      VH_CUDA_TRY(cudaMalloc(&A.val, std::max<int64_t>(1, A.nnz) * sizeof(double)));
      VH_CUDA_TRY(cudaMemcpyAsync(A.rowptr, hA.rp.data(), (nrows + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st));
      if (A.nnz) {
        VH_CUDA_TRY(cudaMemcpyAsync(A.col, hA.col.data(), A.nnz * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        VH_CUDA_TRY(cudaMemcpyAsync(A.val, hA.val.data(), A.nnz * sizeof(double), cudaMemcpyHostToDevice, st));
      }
      DevicePool& pool = ctx->pool;
      auto* d_x = static_cast<double2*>(pool.get((size_t)B * std::max<int64_t>(1, ncols) * sizeof(double2)));
      auto* d_y = static_cast<double2*>(pool.get((size_t)B * std::max<int64_t>(1, nrows) * sizeof(double2)));
      if (ncols > 0)
        VH_CUDA_TRY(cudaMemcpy2DAsync(d_x, ncols * sizeof(double2), x, ldx * sizeof(double2), ncols * sizeof(double2),
                                      B, cudaMemcpyHostToDevice, st));
      spmv_batched(A, B, d_x, ncols, 0, d_y, nrows, 0, 0, st);
      if (nrows > 0)
        VH_CUDA_TRY(cudaMemcpy2DAsync(y, ldy * sizeof(double2), d_y, nrows * sizeof(double2), nrows * sizeof(double2),
                                      B, cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
      pool.put(d_x);
      pool.put(d_y);
    } catch (...) {
      A.free_all();
      throw;
    }
    A.free_all();
  });
}

}  // extern "C"
