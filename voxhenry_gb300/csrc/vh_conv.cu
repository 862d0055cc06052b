// FFT convolution with the 7-component circulant Green tensor, batched over RHS.
//
// Restates the FFT part of lse_matvect_mult.m:34-128 (scatter to the L x M x N x 5
// grid, five zero-padded 3-D FFTs to 2L x 2M 2N, 13 distinct tensor products,
// five inverse FFTs, crop, diagonal z/dx {1,1,1,1/6,1/2} term, gather) as five
// passes over HBM:
//   1. fwd-x : gather x_J through the voxel map, FFT along x (input half zero)
//              -> A[b][c][z][y][kx<2L]
//   2. fwd-y : FFT along y (input half zero)          -> B[b][c][z][ky<2M][kx]
//   3. z     : FFT along z, multiply by the tensor spectrum, inverse FFT along z,
//              keep the voxel rows (in place in B).  The 7 tensor values of a point stay
//              in registers while the CTA walks the RHS batch.
//   4. inv-y : inverse FFT along y, keep the voxel rows -> A
//   5. inv-x : inverse FFT along x, keep x<L, add the diagonal term, scatter to y_J.
// Only the bounding box of the voxels in y and z is visited: y in [y0, y0+ny), z in
// [z0, z0+nz) (A and B hold those rows, compact).  Lines outside it are zero on input and
// unused on output, so the result is the same as that of the full padded transform.
// The 1/(8LMN) normalisation of ifftn is folded into the stored tensor; the
// frequency factor j*omega*mu is a per-RHS scalar applied in pass 5.
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "vh_conv.cuh"
#include "vh_conv_passes.cuh"
#include "vh_df.cuh"

namespace vh {

bool fft_factor(int n, FftDesc& d) {
  memset(&d, 0, sizeof(d));
  d.n = n;
  if (n < 2) return false;
  int m = n;
  std::vector<int> r;
  while (m % 8 == 0) { r.push_back(8); m /= 8; }
  while (m % 4 == 0) { r.push_back(4); m /= 4; }
  while (m % 2 == 0) { r.push_back(2); m /= 2; }
  while (m % 3 == 0) { r.push_back(3); m /= 3; }
  while (m % 5 == 0) { r.push_back(5); m /= 5; }
  while (m % 7 == 0) { r.push_back(7); m /= 7; }
  if (m != 1 || (int)r.size() > kMaxStages) return false;
  d.nstages = (int)r.size();
  for (size_t i = 0; i < r.size(); ++i) d.radix[i] = (signed char)r[i];
  return true;
}

// tw[m] = exp(-2 pi i m / n), evaluated in long double and rounded once.
static std::vector<double2> twiddles(int n) {
  std::vector<double2> t(n);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int m = 0; m < n; ++m) {
    // reduce the angle to [0, pi/4] by symmetry for accuracy
    long double a = 2.0L * pi * (long double)m / (long double)n;
    t[m] = make_double2((double)cosl(a), (double)-sinl(a));
  }
  return t;
}

// fN_all (column-major 2L,2M,2N,7) -> internal [ky][kz][k][kx] divided by X*Y*Z
template <typename C>
__global__ void k_tensor_permute(const double2* __restrict__ raw, C* __restrict__ out, int X, int Y, int Z, double s) {
  const int64_t P = (int64_t)X * Y * Z;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < 7 * P; idx += (int64_t)gridDim.x * blockDim.x) {
    // idx over the OUTPUT layout
    const int kx = idx % X;
    const int k = (idx / X) % 7;
    const int kz = (idx / (7 * (int64_t)X)) % Z;
    const int ky = idx / (7 * (int64_t)X * Z);
    const double2 v = raw[kx + (int64_t)X * (ky + (int64_t)Y * (kz + (int64_t)Z * k))];
    out[idx] = to_c(cscale(v, s), C());
  }
}

// max |Re| and max |Im| of each of the 7 components of fN_all (column-major 2L,2M,2N,7): out[2k],
// out[2k+1] as the bit patterns of non-negative doubles (ordered like the values)
__global__ void k_tensor_reim_max(const double2* __restrict__ raw, int64_t P, unsigned long long* out) {
  double mr[7] = {0, 0, 0, 0, 0, 0, 0}, mi[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < 7 * P; idx += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / P);
    const double2 v = raw[idx];
#pragma unroll
    for (int q = 0; q < 7; ++q)
      if (q == k) {
        mr[q] = fmax(mr[q], fabs(v.x));
        mi[q] = fmax(mi[q], fabs(v.y));
      }
  }
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    atomicMax(&out[2 * q], (unsigned long long)__double_as_longlong(mr[q]));
    atomicMax(&out[2 * q + 1], (unsigned long long)__double_as_longlong(mi[q]));
  }
}

// fN_all -> internal [ky][kz][k][kx] layout, divided by X*Y*Z, one float per component: the real
// part of components 0, 3, 5, 6 and the imaginary part of 1, 2, 4
__global__ void k_tensor_permute_ri(const double2* __restrict__ raw, float* __restrict__ out, int X, int Y, int Z,
                                    double s) {
  const int64_t P = (int64_t)X * Y * Z;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < 7 * P; idx += (int64_t)gridDim.x * blockDim.x) {
    const int kx = idx % X;
    const int k = (idx / X) % 7;
    const int kz = (idx / (7 * (int64_t)X)) % Z;
    const int ky = idx / (7 * (int64_t)X * Z);
    const double2 v = raw[kx + (int64_t)X * (ky + (int64_t)Y * (kz + (int64_t)Z * k))];
    out[idx] = (float)((k == 1 || k == 2 || k == 4 ? v.y : v.x) * s);
  }
}

// ------------------------------------------------------------------------------------------
void conv_plan_create(ConvPlan& p, int L, int M, int N, double dx, const double2* fN_all_dev, int64_t nv,
                      const int64_t* idxS_host, bool want32, cudaStream_t st) {
  p.L = L; p.M = M; p.N = N; p.X = 2 * L; p.Y = 2 * M; p.Z = 2 * N; p.nv = nv; p.dx = dx;
  VH_REQUIRE(fft_factor(p.X, p.fx) && fft_factor(p.Y, p.fy) && fft_factor(p.Z, p.fz), ERR_UNSUPPORTED,
             "padded grid dimensions must factor into 2, 3, 5 and 7");
  VH_REQUIRE(p.X <= 4096 && p.Y <= 4096 && p.Z <= 512, ERR_UNSUPPORTED, "padded grid dimension too large");
  // voxel map
  const int64_t lmn = p.lmn();
  std::vector<int32_t> vm(lmn, -1);
  for (int64_t v = 0; v < nv; ++v) {
    const int64_t li = idxS_host[v] - 1;
    VH_REQUIRE(li >= 0 && li < lmn, ERR_BAD_ARG, "idxS entry out of range");
    VH_REQUIRE(v == 0 || idxS_host[v] > idxS_host[v - 1], ERR_BAD_ARG, "idxS must be strictly increasing");
    vm[li] = (int32_t)v;
  }
  int ylo = M, yhi = -1, zlo = N, zhi = -1;
  for (int64_t v = 0; v < nv; ++v) {
    const int64_t li = idxS_host[v] - 1;
    const int y = (int)((li / L) % M), z = (int)(li / ((int64_t)L * M));
    ylo = std::min(ylo, y); yhi = std::max(yhi, y);
    zlo = std::min(zlo, z); zhi = std::max(zhi, z);
  }
  p.y0 = nv ? ylo : 0; p.ny = nv ? yhi - ylo + 1 : 0;
  p.z0 = nv ? zlo : 0; p.nz = nv ? zhi - zlo + 1 : 0;
  VH_CUDA_TRY(cudaMalloc(&p.vmap, lmn * sizeof(int32_t)));
  VH_CUDA_TRY(cudaMemcpyAsync(p.vmap, vm.data(), lmn * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  // twiddles
  const int dims[3] = {p.X, p.Y, p.Z};
  for (int a = 0; a < 3; ++a) {
    auto t = twiddles(dims[a]);
    VH_CUDA_TRY(cudaMalloc(&p.tw64[a], dims[a] * sizeof(double2)));
    VH_CUDA_TRY(cudaMemcpy(p.tw64[a], t.data(), dims[a] * sizeof(double2), cudaMemcpyHostToDevice));
    std::vector<float2> tf(dims[a]);
    for (int i = 0; i < dims[a]; ++i) tf[i] = make_float2((float)t[i].x, (float)t[i].y);
    VH_CUDA_TRY(cudaMalloc(&p.tw32[a], dims[a] * sizeof(float2)));
    VH_CUDA_TRY(cudaMemcpy(p.tw32[a], tf.data(), dims[a] * sizeof(float2), cudaMemcpyHostToDevice));
  }
  // tensor
  const int64_t P = p.points();
  const double s = 1.0 / (double)P;
  VH_CUDA_TRY(cudaMalloc(&p.tens64, 7 * P * sizeof(double2)));
  k_tensor_permute<double2><<<1024, 256, 0, st>>>(fN_all_dev, p.tens64, p.X, p.Y, p.Z, s);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  // real/imaginary check of each component over the whole spectrum (the complex64 and double-float
  // products use the one-value-per-component tensor when it holds)
  {
    unsigned long long* d_mx = nullptr;
    VH_CUDA_TRY(cudaMalloc(&d_mx, 14 * sizeof(unsigned long long)));
    VH_CUDA_TRY(cudaMemsetAsync(d_mx, 0, 14 * sizeof(unsigned long long), st));
    k_tensor_reim_max<<<1024, 256, 0, st>>>(fN_all_dev, P, d_mx);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    unsigned long long hmx[14];
    VH_CUDA_TRY(cudaMemcpyAsync(hmx, d_mx, sizeof(hmx), cudaMemcpyDeviceToHost, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(d_mx);
    bool ri = true;
    for (int k = 0; k < 7; ++k) {
      double re, im;
      std::memcpy(&re, &hmx[2 * k], sizeof(double));
      std::memcpy(&im, &hmx[2 * k + 1], sizeof(double));
      const bool imag_kind = (k == 1 || k == 2 || k == 4);
      ri = ri && (imag_kind ? re <= 1e-9 * im : im <= 1e-9 * re);
    }
    p.ri = ri;
  }
  if (want32) {
    VH_CUDA_TRY(cudaMalloc(&p.tens32, 7 * P * sizeof(float2)));
    k_tensor_permute<float2><<<1024, 256, 0, st>>>(fN_all_dev, p.tens32, p.X, p.Y, p.Z, s);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    if (p.ri) {
      VH_CUDA_TRY(cudaMalloc(&p.tens32ri, 7 * P * sizeof(float)));
      k_tensor_permute_ri<<<1024, 256, 0, st>>>(fN_all_dev, p.tens32ri, p.X, p.Y, p.Z, s);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    }
  }
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

// the double-float real/imaginary tensor of PREC_DF from tens64 (layout [ky][kz][k][kx]): the real
// part of components 0, 3, 5, 6 and the imaginary part of 1, 2, 4, as pairs (once per plan)
__global__ void k_tensor_to_df_ri(const double2* __restrict__ in, dfloat* __restrict__ out, int X, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)((i / X) % 7);
    out[i] = dfloat((k == 1 || k == 2 || k == 4) ? in[i].y : in[i].x);
  }
}

static void ensure_df_tensor(ConvPlan& p, cudaStream_t st) {
  if (p.tensdf) return;
  const int64_t n = 7 * p.points();
  VH_CUDA_TRY(cudaMalloc(&p.tensdf, n * sizeof(dfloat)));
  k_tensor_to_df_ri<<<1024, 256, 0, st>>>(p.tens64, static_cast<dfloat*>(p.tensdf), p.X, n);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  void** dst[3] = {&p.twxdf, &p.twydf, &p.twdf};
  const int dims[3] = {p.X, p.Y, p.Z};
  std::vector<std::vector<dcomplex>> td(3);
  for (int a = 0; a < 3; ++a) {
    const auto t = twiddles(dims[a]);
    td[a].resize(dims[a]);
    for (int i = 0; i < dims[a]; ++i) td[a][i] = dcomplex{dfloat(t[i].x), dfloat(t[i].y)};
    VH_CUDA_TRY(cudaMalloc(dst[a], dims[a] * sizeof(dcomplex)));
    VH_CUDA_TRY(cudaMemcpyAsync(*dst[a], td[a].data(), dims[a] * sizeof(dcomplex), cudaMemcpyHostToDevice, st));
  }
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

void conv_plan_destroy(ConvPlan& p) {
  cudaFree(p.vmap);
  cudaFree(p.tens64);
  cudaFree(p.tens32);
  cudaFree(p.tens32ri);
  cudaFree(p.tensdf);
  cudaFree(p.tensz);
  cudaFree(p.twdf);
  cudaFree(p.twxdf);
  cudaFree(p.twydf);
  for (int a = 0; a < 3; ++a) { cudaFree(p.tw64[a]); cudaFree(p.tw32[a]); }
  cudaFree(p.scratchA);
  cudaFree(p.scratchB);
  p = ConvPlan{};
}

void conv_plan_reserve(ConvPlan& p, int B, Prec prec) {
  const size_t cs = prec == PREC_FP32 ? sizeof(float2) : sizeof(double2);
  const size_t needA = (size_t)B * 5 * p.nz * p.ny * p.X * cs;
  const size_t needB = (size_t)B * 5 * p.nz * p.Y * p.X * cs;
  if (needA > p.scratch_bytes_A) {
    cudaFree(p.scratchA);
    p.scratchA = nullptr;
    p.scratch_bytes_A = 0;
    VH_CUDA_TRY(cudaMalloc(&p.scratchA, needA));
    p.scratch_bytes_A = needA;
  }
  if (needB > p.scratch_bytes_B) {
    cudaFree(p.scratchB);
    p.scratchB = nullptr;
    p.scratch_bytes_B = 0;
    VH_CUDA_TRY(cudaMalloc(&p.scratchB, needB));
    p.scratch_bytes_B = needB;
  }
}

// ---------------------------------------------------------------------------- plain 3-D FFT
// Forward FFT along one axis of a column-major array, in place.  Element (i, col) of plane p
// sits at data[p * n * inner + i * inner + col]; a CTA takes `tx` consecutive columns.
__global__ void k_fft_axis_inplace(double2* data, int64_t inner, FftDesc fd, const double2* __restrict__ twg, int tx,
                                   bool contiguous) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = fd.n;
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* b0 = tw + n;
  double2* b1 = b0 + n * tx;
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = twg[i];
  const int64_t plane = blockIdx.y;
  const int64_t c0 = (int64_t)blockIdx.x * tx;
  double2* base = data + plane * n * inner;
  if (contiguous) {   // lines are contiguous (inner == 1 axis is x): column = line index
    for (int t = threadIdx.x; t < n * tx; t += blockDim.x) {
      const int line = t / n, i = t % n;
      const int64_t col = c0 + line;
      b0[line * n + i] = (col < inner) ? base[col * n + i] : make_double2(0.0, 0.0);
    }
  } else {
    for (int t = threadIdx.x; t < n * tx; t += blockDim.x) {
      const int line = t % tx, i = t / tx;
      const int64_t col = c0 + line;
      b0[i * tx + line] = (col < inner) ? base[(int64_t)i * inner + col] : make_double2(0.0, 0.0);
    }
  }
  __syncthreads();
  double2* r = contiguous ? fft_lines<-1>(b0, b1, tw, fd, 1, n, tx, true) : fft_lines<-1>(b0, b1, tw, fd, tx, 1, tx, false);
  if (contiguous) {
    for (int t = threadIdx.x; t < n * tx; t += blockDim.x) {
      const int line = t / n, i = t % n;
      const int64_t col = c0 + line;
      if (col < inner) base[col * n + i] = r[line * n + i];
    }
  } else {
    for (int t = threadIdx.x; t < n * tx; t += blockDim.x) {
      const int line = t % tx, i = t / tx;
      const int64_t col = c0 + line;
      if (col < inner) base[(int64_t)i * inner + col] = r[i * tx + line];
    }
  }
}

void fft3d_forward_inplace(double2* data, int X, int Y, int Z, int batch, cudaStream_t st) {
  const int dims[3] = {X, Y, Z};
  for (int a = 0; a < 3; ++a) {
    FftDesc fd;
    VH_REQUIRE(fft_factor(dims[a], fd), ERR_UNSUPPORTED, "tensor grid dimensions must factor into 2, 3, 5 and 7");
    VH_REQUIRE(dims[a] <= 4096, ERR_UNSUPPORTED, "tensor grid dimension too large");
  }
  for (int a = 0; a < 3; ++a) {
    const int n = dims[a];
    FftDesc fd;
    fft_factor(n, fd);
    auto t = twiddles(n);
    double2* tw = nullptr;
    VH_CUDA_TRY(cudaMalloc(&tw, n * sizeof(double2)));
    VH_CUDA_TRY(cudaMemcpyAsync(tw, t.data(), n * sizeof(double2), cudaMemcpyHostToDevice, st));
    int64_t inner, planes;
    bool contiguous = (a == 0);
    int tx;
    if (a == 0) {            // lines along x: "inner" counts the lines of one plane set
      inner = (int64_t)Y * Z * batch;
      planes = 1;
      tx = std::max(1, std::min(16, 2048 / n));
    } else if (a == 1) {
      inner = X;
      planes = (int64_t)Z * batch;
      tx = std::max(1, std::min(16, 4096 / n));
    } else {
      inner = (int64_t)X * Y;
      planes = batch;
      tx = std::max(1, std::min(16, 4096 / n));
    }
    const size_t sm = (size_t)(n + 2 * n * tx) * sizeof(double2);
    allow_dyn_smem(k_fft_axis_inplace, sm);
    dim3 grid((unsigned)ceil_div(inner, tx), (unsigned)planes);
    k_fft_axis_inplace<<<grid, kPassThreads, sm, st>>>(data, inner, fd, tw, tx, contiguous);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(tw);
  }
}

void conv_apply(ConvPlan& p, Prec prec, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st) {
  const ConvTuning& t = p.tune[prec];
  const int w = (t.max_rhs > 0 && t.max_rhs < B) ? t.max_rhs : B;   // right-hand sides per launch sequence
  conv_plan_reserve(p, w, prec);
  if (prec == PREC_DF && conv_df_supported(p)) ensure_df_tensor(p, st);
  p.y_variant_now = t.y_variant;
  p.z_variant_now = t.z_variant;
  // the automatic choices of complex64 (the faster variants on every measured grid): warp-per-line x
  // passes where X fits, the Toeplitz z-pass where the box is short enough and the table builds
  p.x_variant_now = prec != PREC_FP32 ? 0 : (t.x_variant == 0 ? (xpass_warp_ok(p) ? 1 : 0) : (t.x_variant == 1 ? 1 : 0));
  if (prec == PREC_FP32 && t.z_variant == 0 && p.nz <= kZtoepMaxRows && ztoep_build(p, st)) p.z_variant_now = 3;
  if (t.z_variant == 3 && (prec == PREC_FP64 || !ztoep_build(p, st))) p.z_variant_now = 0;
  for (int b0 = 0; b0 < B; b0 += w) {
    const int nb = std::min(w, B - b0);
    const double2* xb = x + (int64_t)b0 * ldx;
    double2* yb = y + (int64_t)b0 * ldy;
    const double2* zb = zdiag + (int64_t)b0 * zstride;
    if (prec == PREC_FP32)
      conv_apply_c64(p, nb, xb, ldx, yb, ldy, scale + b0, zb, zstride, st);
    else if (prec == PREC_DF && conv_df_supported(p))
      conv_apply_df(p, nb, xb, ldx, yb, ldy, scale + b0, zb, zstride, st);
    else
      conv_apply_t<double>(p, nb, xb, ldx, yb, ldy, scale + b0, zb, zstride, st);
  }
  p.y_variant_now = 0;
  p.z_variant_now = 0;
  p.x_variant_now = 0;
}

void conv_scratch_bytes(const ConvPlan& p, Prec prec, size_t& a_per_rhs, size_t& b_per_rhs) {
  const size_t cs = prec == PREC_FP32 ? sizeof(float2) : sizeof(double2);
  a_per_rhs = (size_t)5 * p.nz * p.ny * p.X * cs;
  b_per_rhs = (size_t)5 * p.nz * p.Y * p.X * cs;
}

void conv_apply_scratch(const ConvPlan& p, Prec prec, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                        const double2* scale, const double2* zdiag, int64_t zstride, void* scratchA, void* scratchB,
                        cudaStream_t st) {
  VH_REQUIRE(((uintptr_t)scratchA | (uintptr_t)scratchB) % 16 == 0, ERR_BAD_ARG, "FFT scratch must be 16-byte aligned");
  size_t a1, b1;
  conv_scratch_bytes(p, prec, a1, b1);
  ConvPlan q = p;   // shallow view of the plan with the caller's scratch; owns nothing
  q.y_variant_now = 0;   // the automatic pass choices
  q.z_variant_now = 0;
  q.x_variant_now = prec == PREC_FP32 && xpass_warp_ok(p) ? 1 : 0;   // allocates nothing
  q.scratchA = scratchA;
  q.scratchB = scratchB;
  q.scratch_bytes_A = a1 * B;
  q.scratch_bytes_B = b1 * B;
  if (prec == PREC_FP32)
    conv_apply_c64(q, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
  else if (prec == PREC_DF && p.tensdf && conv_df_supported(p))   // only if the plan holds its tables
    conv_apply_df(q, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
  else
    conv_apply_t<double>(q, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
}

}  // namespace vh
