// Panel numbering and the incidence matrix on the device (the setup of every request in the serving
// loop): lse_generate_panelIDs.m:25-172 and lse_compute_Ae_matrix.m:205-264.
//
// Panel ids by scan: along axis a the reference visits the grid with a innermost (x panels: x, then
// y, then z; y panels: y, then z, then x; z panels: z, then x, then y) and keeps a running index that
// grows by one at every non-empty voxel and by one more where the voxel's run along a ends (the next
// cell is empty or outside the grid).  A voxel's two node ids along a are therefore
//   offset_a + 1 + (sum over the cells before it in that order of w),  and that plus one,
// with w = [non-empty] + [non-empty and the run ends]: one weight kernel, one exclusive prefix sum and
// one assignment kernel per axis.  The ids are those of the sequential loop exactly.
// Ae by closed form: column (c, v) has 2, 2, 2, 4 or 6 entries (c = Jx, Jy, Jz, J2D, J3D) whose rows
// are the voxel's panel ids, in increasing order, and whose values are the fixed coefficients.
#include <vector>

#include "../../include/voxhenry_gpu.h"
#include "vh_internal.cuh"

namespace vh {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 2 * kScanThreads;   // elements per scan block

__global__ void k_voxel_map(const int64_t* __restrict__ idxS, int64_t nv, int64_t lmn, int32_t* __restrict__ vnum,
                            int* __restrict__ bad) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = idxS[v] - 1;
    const bool ok = li >= 0 && li < lmn && (v == 0 || idxS[v] > idxS[v - 1]);
    if (ok)
      vnum[li] = (int32_t)v;
    else
      atomicExch(bad, 1);
  }
}

// the (x, y, z) cell at position s of axis a's scan order (a innermost, then o2, then o1)
__device__ __forceinline__ void scan_cell(int64_t s, int a, int L, int M, int N, int& x, int& y, int& z) {
  const int dims[3] = {L, M, N};
  const int o2 = a == 0 ? 1 : (a == 1 ? 2 : 0);
  const int da = dims[a], d2 = dims[o2];
  int c[3];
  c[a] = (int)(s % da);
  const int64_t r = s / da;
  c[o2] = (int)(r % d2);
  c[a == 0 ? 2 : (a == 1 ? 0 : 1)] = (int)(r / d2);
  x = c[0];
  y = c[1];
  z = c[2];
}

__global__ void k_panel_weights(const int32_t* __restrict__ vnum, int L, int M, int N, int a, int64_t* __restrict__ w) {
  const int64_t lmn = (int64_t)L * M * N;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < lmn; s += (int64_t)gridDim.x * blockDim.x) {
    int x, y, z;
    scan_cell(s, a, L, M, N, x, y, z);
    const int64_t li = x + (int64_t)L * (y + (int64_t)M * z);
    int64_t wt = 0;
    if (vnum[li] >= 0) {
      int d[3] = {x, y, z};
      const int dims[3] = {L, M, N};
      d[a] += 1;
      const bool end = d[a] >= dims[a] || vnum[d[0] + (int64_t)L * (d[1] + (int64_t)M * d[2])] < 0;
      wt = end ? 2 : 1;
    }
    w[s] = wt;
  }
}

// exclusive prefix sums of kScanItems-element blocks in place; block totals to sums[blockIdx.x]
__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(int64_t* __restrict__ d, int64_t n,
                                                              int64_t* __restrict__ sums) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanItems;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int64_t i0 = base + 2 * t;
  const int64_t a = i0 < n ? d[i0] : 0, b = i0 + 1 < n ? d[i0 + 1] : 0;
  int64_t v = a + b;   // inclusive scan of the thread pairs
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) warp_tot[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int64_t s = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    warp_tot[lane] = s;   // inclusive over warps
  }
  __syncthreads();
  const int64_t before = v - (a + b) + (warp > 0 ? warp_tot[warp - 1] : 0);
  if (i0 < n) d[i0] = before;
  if (i0 + 1 < n) d[i0 + 1] = before + a;
  if (t == kScanThreads - 1) sums[blockIdx.x] = warp_tot[kScanThreads / 32 - 1];
}

__global__ void k_scan_add(int64_t* __restrict__ d, int64_t n, const int64_t* __restrict__ offs) {
  const int64_t i = blockIdx.x * (int64_t)kScanItems + threadIdx.x;
  const int64_t o = offs[blockIdx.x];
  if (i < n) d[i] += o;
  if (i + kScanThreads < n) d[i + kScanThreads] += o;
}

// exclusive prefix sum of d[0..n) in place; returns the total
int64_t exclusive_scan(int64_t* d, int64_t n, cudaStream_t st) {
  if (n <= 0) return 0;
  const int64_t nb = ceil_div(n, kScanItems);
  int64_t* sums = nullptr;
  VH_CUDA_TRY(cudaMalloc(&sums, (size_t)std::max<int64_t>(nb, 1) * sizeof(int64_t)));
  int64_t total = 0;
  try {
    k_scan_blocks<<<(unsigned)nb, kScanThreads, 0, st>>>(d, n, sums);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    if (nb > 1) {
      total = exclusive_scan(sums, nb, st);   // block offsets (recursive for very large grids)
      k_scan_add<<<(unsigned)nb, kScanThreads, 0, st>>>(d, n, sums);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    } else {
      VH_CUDA_TRY(cudaMemcpyAsync(&total, sums, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    }
  } catch (...) {
    cudaFree(sums);
    throw;
  }
  cudaFree(sums);
  return total;
}

__global__ void k_panel_assign(const int32_t* __restrict__ vnum, const int64_t* __restrict__ excl, int L, int M,
                               int N, int a, int64_t offset, int64_t nv, int64_t* __restrict__ apid) {
  const int64_t lmn = (int64_t)L * M * N;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < lmn; s += (int64_t)gridDim.x * blockDim.x) {
    int x, y, z;
    scan_cell(s, a, L, M, N, x, y, z);
    const int32_t v = vnum[x + (int64_t)L * (y + (int64_t)M * z)];
    if (v < 0) continue;
    const int64_t left = offset + 1 + excl[s];
    apid[v + nv * (2 * a)] = left;
    apid[v + nv * (2 * a + 1)] = left + 1;
  }
}

__constant__ double c_coef[5][6] = {{-1, 1, 0, 0, 0, 0},          {0, 0, -1, 1, 0, 0},        {0, 0, 0, 0, -1, 1},
                                    {0.5, 0.5, -0.5, -0.5, 0, 0}, {0.5, 0.5, 0.5, 0.5, -1, -1}};

// column (c, v) of Ae: entries at base_c + v nnz_c, panel ids in increasing p order
__global__ void k_incidence(const int64_t* __restrict__ apid, int64_t nv, int64_t* __restrict__ jc,
                            int64_t* __restrict__ ir, double* __restrict__ pr) {
  const int nnz_c[5] = {2, 2, 2, 4, 6};
  const int base_c[5] = {0, 2, 4, 6, 10};   // times nv
  for (int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; col < 5 * nv;
       col += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(col / nv);
    const int64_t v = col - (int64_t)c * nv;
    const int64_t start = base_c[c] * nv + v * nnz_c[c];
    jc[col + 1] = start + nnz_c[c];
    if (col == 0) jc[0] = 0;
    int64_t k = start;
    for (int p = 0; p < 6; ++p) {
      const double cf = c_coef[c][p];
      if (cf != 0.0) {
        ir[k] = apid[v + nv * p] - 1;
        pr[k] = cf;
        ++k;
      }
    }
  }
}

template <typename T>
struct DevArr {
  T* p = nullptr;
  explicit DevArr(size_t n) { VH_CUDA_TRY(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T))); }
  ~DevArr() { cudaFree(p); }
};

}  // namespace
}  // namespace vh

using namespace vh;

extern "C" {

vh_status vh_setup_device(vh_ctx* ctx, int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t* all_panels_ids,
                          int64_t* num_nodes, int64_t* Ae_jc, int64_t* Ae_ir, double* Ae_pr) {
  if (!ctx) return VH_ERR_BAD_ARG;
  try {
    VH_REQUIRE(L >= 1 && M >= 1 && N >= 1 && nv >= 0 && num_nodes && (nv == 0 || (idxS && all_panels_ids)),
               ERR_BAD_ARG, "bad arguments");
    const int64_t lmn = (int64_t)L * M * N;
    VH_REQUIRE(nv <= lmn && lmn < (1LL << 31), ERR_BAD_ARG, "nv exceeds the grid or the grid is too large");
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    *num_nodes = 0;
    if (nv == 0) return VH_OK;
    DevArr<int64_t> d_idx(nv), d_apid(6 * nv), w(lmn);
    DevArr<int32_t> vnum(lmn);
    DevArr<int> bad(1);
    VH_CUDA_TRY(cudaMemcpyAsync(d_idx.p, idxS, nv * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    VH_CUDA_TRY(cudaMemsetAsync(vnum.p, 0xff, lmn * sizeof(int32_t), st));   // -1: empty
    VH_CUDA_TRY(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    const unsigned gv = (unsigned)std::min<int64_t>(4096, ceil_div(nv, 256));
    const unsigned gl = (unsigned)std::min<int64_t>(4096, ceil_div(lmn, 256));
    k_voxel_map<<<gv, 256, 0, st>>>(d_idx.p, nv, lmn, vnum.p, bad.p);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    int h_bad = 0;
    VH_CUDA_TRY(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    VH_REQUIRE(!h_bad, ERR_BAD_ARG, "idxS must be strictly increasing 1-based indices into the grid");
    int64_t offset = 0;
    for (int a = 0; a < 3; ++a) {
      k_panel_weights<<<gl, 256, 0, st>>>(vnum.p, L, M, N, a, w.p);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      const int64_t np = exclusive_scan(w.p, lmn, st);   // nodes along this axis
      k_panel_assign<<<gl, 256, 0, st>>>(vnum.p, w.p, L, M, N, a, offset, nv, d_apid.p);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      offset += np;
    }
    *num_nodes = offset;
    VH_CUDA_TRY(cudaMemcpyAsync(all_panels_ids, d_apid.p, 6 * nv * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    if (Ae_jc && Ae_ir && Ae_pr) {
      DevArr<int64_t> jc(5 * nv + 1), ir(16 * nv);
      DevArr<double> pr(16 * nv);
      k_incidence<<<gv, 256, 0, st>>>(d_apid.p, nv, jc.p, ir.p, pr.p);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      VH_CUDA_TRY(cudaMemcpyAsync(Ae_jc, jc.p, (5 * nv + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaMemcpyAsync(Ae_ir, ir.p, 16 * nv * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaMemcpyAsync(Ae_pr, pr.p, 16 * nv * sizeof(double), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    } else {
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return VH_OK;
  } catch (const Error& e) {
    ctx->last_error = e.msg;
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {
    ctx->last_error = "host allocation failed";
    return VH_ERR_OOM;
  }
}

}  // extern "C"
