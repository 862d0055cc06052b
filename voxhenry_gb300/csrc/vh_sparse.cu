// Sparse incidence products Ae*J and Ae^T*phi of lse_matvect_mult.m:138-140 and
// lse_sparse_precon_multiply.m:84-88, batched over right-hand sides.
#include <algorithm>
#include <vector>

#include "vh_internal.cuh"

namespace vh {

// One thread per (row, rhs).  Rows of Ae have <= 6 entries (a panel touches <= 2 voxels,
// 3 current components each); rows of Ae^T have 2..6 (lse_compute_Ae_matrix.m:205-262).
__global__ void k_spmv(int64_t nrows, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                       const double* __restrict__ val, const double2* __restrict__ x, int64_t ldx, int64_t xoff,
                       double2* __restrict__ y, int64_t ldy, int64_t yoff, int mode) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = blockIdx.y;
  if (r >= nrows) return;
  const double2* xb = x + b * ldx + xoff;
  double2 acc = make_double2(0.0, 0.0);
  for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
    const double a = val[k];
    const double2 v = xb[col[k]];
    acc.x = fma(a, v.x, acc.x);
    acc.y = fma(a, v.y, acc.y);
  }
  double2* yp = y + b * ldy + yoff + r;
  if (mode == 0) {
    *yp = acc;
  } else if (mode > 0) {
    double2 t = *yp;
    *yp = make_double2(t.x + acc.x, t.y + acc.y);
  } else {
    double2 t = *yp;
    *yp = make_double2(t.x - acc.x, t.y - acc.y);
  }
}

void spmv_batched(const Csr& A, int B, const double2* x, int64_t ldx, int64_t xoff, double2* y, int64_t ldy,
                  int64_t yoff, int mode, cudaStream_t st) {
  if (A.nrows == 0 || B == 0) return;
  dim3 grid((unsigned)ceil_div(A.nrows, 256), (unsigned)B);
  k_spmv<<<grid, 256, 0, st>>>(A.nrows, A.rowptr, A.col, A.val, x, ldx, xoff, y, ldy, yoff, mode);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

static void upload_csr(int64_t nrows, int64_t ncols, const std::vector<int32_t>& rp, const std::vector<int32_t>& col,
                       const std::vector<double>& val, Csr& out, cudaStream_t st) {
  out.nrows = nrows;
  out.ncols = ncols;
  out.nnz = (int64_t)col.size();
  VH_CUDA_TRY(cudaMalloc(&out.rowptr, (nrows + 1) * sizeof(int32_t)));
  VH_CUDA_TRY(cudaMalloc(&out.col, std::max<int64_t>(1, out.nnz) * sizeof(int32_t)));
  VH_CUDA_TRY(cudaMalloc(&out.val, std::max<int64_t>(1, out.nnz) * sizeof(double)));
  VH_CUDA_TRY(cudaMemcpyAsync(out.rowptr, rp.data(), (nrows + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  if (out.nnz) {
    VH_CUDA_TRY(cudaMemcpyAsync(out.col, col.data(), out.nnz * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    VH_CUDA_TRY(cudaMemcpyAsync(out.val, val.data(), out.nnz * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

void csc_to_host(int64_t nrow, int64_t ncol, const int64_t* jc, const int64_t* ir, const double* pr, HostCsr& hA,
                 HostCsr& hAT) {
  const int64_t nnz = jc[ncol];
  VH_REQUIRE(jc[0] == 0 && nnz >= 0 && nnz < (1LL << 31), ERR_BAD_ARG, "bad CSC column offsets");
  for (int64_t j = 0; j < ncol; ++j)
    VH_REQUIRE(jc[j + 1] >= jc[j], ERR_BAD_ARG, "CSC column offsets must be non-decreasing");
  // CSC of A is CSR of A^T
  hAT.rp.assign(ncol + 1, 0);
  hAT.col.assign(nnz, 0);
  hAT.val.assign(nnz, 0.0);
  for (int64_t j = 0; j <= ncol; ++j) hAT.rp[j] = (int32_t)jc[j];
  for (int64_t k = 0; k < nnz; ++k) {
    VH_REQUIRE(ir[k] >= 0 && ir[k] < nrow, ERR_BAD_ARG, "CSC row index out of range");
    hAT.col[k] = (int32_t)ir[k];
    hAT.val[k] = pr[k];
  }
  // transpose -> CSR of A
  hA.rp.assign(nrow + 1, 0);
  hA.col.assign(nnz, 0);
  hA.val.assign(nnz, 0.0);
  for (int64_t k = 0; k < nnz; ++k) hA.rp[ir[k] + 1]++;
  for (int64_t r = 0; r < nrow; ++r) hA.rp[r + 1] += hA.rp[r];
  std::vector<int32_t> pos(hA.rp.begin(), hA.rp.end() - 1);
  for (int64_t j = 0; j < ncol; ++j)
    for (int64_t k = jc[j]; k < jc[j + 1]; ++k) {
      const int32_t q = pos[ir[k]]++;
      hA.col[q] = (int32_t)j;
      hA.val[q] = pr[k];
    }
}

void csc_upload(int64_t nrow, int64_t ncol, const int64_t* jc, const int64_t* ir, const double* pr, Csr& A, Csr& AT,
                HostCsr& hA, HostCsr& hAT, cudaStream_t st) {
  csc_to_host(nrow, ncol, jc, ir, pr, hA, hAT);
  upload_csr(nrow, ncol, hA.rp, hA.col, hA.val, A, st);
  upload_csr(ncol, nrow, hAT.rp, hAT.col, hAT.val, AT, st);
}

}  // namespace vh
