// Passes 1 and 5 of the complex64 FFT convolution with one warp per line (the autotuner's x variant 1)
// for padded x lengths X = 32 R1 in {256, 512, 1024}: the x-transform of a line as R1-point transforms
// in registers (lane n1 holds the elements n1 + 32 n2), a twiddle, one transpose through the warp's
// own shared memory, and 32-point transforms in registers, with no block-wide barrier.  A warp takes
// 32 / R1 lines, so that every lane runs one 32-point transform.
//
//   A[k2 + R1 k1] = sum_n1 W32^(n1 k1) W^(n1 k2) sum_n2 x[n1 + 32 n2] W_R1^(n2 k2),   W = e^(-2 pi i / X)
//
// Forward: the line's upper half (n >= L = X / 2) is zero and its first stage is pruned.  Inverse: the
// same with conjugate twiddles and roles swapped (input index j1 + 32 j2, output n2 + R1 n1); only the
// rows n < L are formed, then the epilogue of the matvec (scale conv + c_k / dx z x) is applied to the
// voxels of the line.  The operations are those of the shared-memory passes (k_fwd_x / k_inv_x) in
// another order, so the products agree to complex64 rounding.
#include "vh_conv.cuh"
#include "vh_fft.cuh"

namespace vh {
namespace {

constexpr int kXwWarps = 4;

struct XwLine {
  int64_t vbase, xoff;
  int b, c;
  bool valid;
};

__device__ __forceinline__ XwLine xw_decode(int64_t gl, int64_t nlines, int L, int M, int y0, int ny, int z0, int nz,
                                            int64_t ld, int64_t nv) {
  XwLine q;
  q.valid = gl < nlines;
  if (!q.valid) gl = 0;
  const int64_t y = y0 + gl % ny;
  const int64_t z = z0 + (gl / ny) % nz;
  q.c = (int)((gl / ((int64_t)ny * nz)) % 5);
  q.b = (int)(gl / ((int64_t)ny * nz * 5));
  q.vbase = (int64_t)L * (y + (int64_t)M * z);
  q.xoff = (int64_t)q.b * ld + (int64_t)q.c * nv;
  return q;
}

template <int R1>
__global__ void __launch_bounds__(kXwWarps * 32)
    k_fwd_x_warp(const double2* __restrict__ xin, int64_t ldx, const int32_t* __restrict__ vmap, int L, int M, int y0,
                 int ny, int z0, int nz, int64_t nv, int64_t nlines, float2* __restrict__ A,
                 const float2* __restrict__ twg) {
  constexpr int X = 32 * R1, LW = 32 / R1, H = R1 / 2;
  __shared__ float2 tw[X];
  __shared__ float2 S[kXwWarps][32 * 33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = twg[i];
  __syncthreads();
  const int64_t l0 = ((int64_t)blockIdx.x * kXwWarps + warp) * LW;
  if (l0 >= nlines) return;
  float2* Sw = S[warp];
#pragma unroll
  for (int l = 0; l < LW; ++l) {
    const XwLine q = xw_decode(l0 + l, nlines, L, M, y0, ny, z0, nz, ldx, nv);
    float2 v[R1];
#pragma unroll
    for (int m = 0; m < R1; ++m) v[m] = make_float2(0.0f, 0.0f);
    if (q.valid) {
#pragma unroll
      for (int m = 0; m < H; ++m) {   // n = lane + 32 m < L
        const int32_t vid = vmap[q.vbase + lane + 32 * m];
        if (vid >= 0) v[m] = to_c(xin[q.xoff + vid], float2());
      }
    }
    dif_pruned<X, R1, H, -1>(v, tw);   // v[p] = Y[k2 = bitrev(p)]
#pragma unroll
    for (int p = 0; p < R1; ++p) {
      const int k2 = bit_reverse<ilog2c(R1)>(p);
      const float2 w = tw[(lane * k2) & (X - 1)];
      Sw[(l * R1 + k2) * 33 + lane] = cmul(v[p], w);
    }
  }
  __syncwarp();
  const int l = lane / R1, k2 = lane % R1;
  float2 u[32];
#pragma unroll
  for (int n1 = 0; n1 < 32; ++n1) u[n1] = Sw[lane * 33 + n1];
  dif_pruned<X, 32, 32, -1>(u, tw);   // u[p] = A[k2 + R1 bitrev(p)]
  if (l0 + l < nlines) {
    float2* out = A + (l0 + l) * X + k2;
#pragma unroll
    for (int p = 0; p < 32; ++p) out[R1 * bit_reverse<5>(p)] = u[p];
  }
}

template <int R1>
__global__ void __launch_bounds__(kXwWarps * 32)
    k_inv_x_warp(const float2* __restrict__ A, const int32_t* __restrict__ vmap, int L, int M, int y0, int ny, int z0,
                 int nz, int64_t nv, int64_t nlines, const double2* __restrict__ xin, int64_t ldx,
                 double2* __restrict__ yout, int64_t ldy, const double2* __restrict__ scale,
                 const double2* __restrict__ zdiag, int64_t zstride, double inv_dx, const float2* __restrict__ twg) {
  constexpr int X = 32 * R1, LW = 32 / R1;
  __shared__ float2 tw[X];
  __shared__ float2 S[kXwWarps][32 * 33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = twg[i];
  __syncthreads();
  const int64_t l0 = ((int64_t)blockIdx.x * kXwWarps + warp) * LW;
  if (l0 >= nlines) return;
  float2* Sw = S[warp];
#pragma unroll
  for (int l = 0; l < LW; ++l) {
    float2 v[R1];
    const bool valid = l0 + l < nlines;
    const float2* in = A + (valid ? l0 + l : l0) * X + lane;
#pragma unroll
    for (int m = 0; m < R1; ++m) v[m] = in[32 * m];   // j = lane + 32 m
    dif_pruned<X, R1, R1, +1>(v, tw);   // v[p] = Z[n2 = bitrev(p)]
#pragma unroll
    for (int p = 0; p < R1; ++p) {
      const int n2 = bit_reverse<ilog2c(R1)>(p);
      const float2 w = tw[(lane * n2) & (X - 1)];
      Sw[(l * R1 + n2) * 33 + lane] = cmulc(v[p], w);
    }
  }
  __syncwarp();
  const int l = lane / R1, n2 = lane % R1;
  float2 u[32];
#pragma unroll
  for (int p = 0; p < 32; ++p) u[p] = Sw[lane * 33 + bit_reverse<5>(p)];   // bit-reversed input
  dit_pruned<X, 32, 16, +1>(u, tw);   // u[n1] = y[n2 + R1 n1], n1 < 16 (n < L)
  const XwLine q = xw_decode(l0 + l, nlines, L, M, y0, ny, z0, nz, ldx, nv);
  if (!q.valid) return;
  const float2 sf = to_c(scale[q.b], float2());
  const float ckf = (float)((q.c < 3 ? 1.0 : (q.c == 3 ? 1.0 / 6.0 : 0.5)) * inv_dx);
#pragma unroll
  for (int n1 = 0; n1 < 16; ++n1) {
    const int i = n2 + R1 * n1;
    const int32_t vid = vmap[q.vbase + i];
    if (vid < 0) continue;
    // the diagonal term in FP32 as k_inv_x does for the complex64 product
    const float2 zf = to_c(zdiag[q.b * zstride + vid], float2());
    const float2 xf = to_c(xin[q.xoff + vid], float2());
    const float2 d = cmul(zf, xf);
    float2 o = cmul(sf, u[n1]);
    o.x = fmaf(ckf, d.x, o.x);
    o.y = fmaf(ckf, d.y, o.y);
    yout[(int64_t)q.b * ldy + (int64_t)q.c * nv + vid] = make_double2((double)o.x, (double)o.y);
  }
}

template <int R1>
void launch_fwd(const ConvPlan& p, int B, const double2* x, int64_t ldx, float2* A, cudaStream_t st) {
  const int64_t lines = (int64_t)p.ny * p.nz * 5 * B;
  const unsigned grid = (unsigned)ceil_div(lines, (int64_t)kXwWarps * (32 / R1));
  k_fwd_x_warp<R1><<<grid, kXwWarps * 32, 0, st>>>(x, ldx, p.vmap, p.L, p.M, p.y0, p.ny, p.z0, p.nz, p.nv, lines, A,
                                                   p.tw32[0]);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

template <int R1>
void launch_inv(const ConvPlan& p, int B, const float2* A, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st) {
  const int64_t lines = (int64_t)p.ny * p.nz * 5 * B;
  const unsigned grid = (unsigned)ceil_div(lines, (int64_t)kXwWarps * (32 / R1));
  k_inv_x_warp<R1><<<grid, kXwWarps * 32, 0, st>>>(A, p.vmap, p.L, p.M, p.y0, p.ny, p.z0, p.nz, p.nv, lines, x, ldx, y,
                                                   ldy, scale, zdiag, zstride, 1.0 / p.dx, p.tw32[0]);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

}  // namespace

bool xpass_warp_ok(const ConvPlan& p) { return p.X == 256 || p.X == 512 || p.X == 1024; }

bool xpass_warp_fwd(const ConvPlan& p, int B, const double2* x, int64_t ldx, float2* A, cudaStream_t st) {
  switch (p.X) {
    case 256: launch_fwd<8>(p, B, x, ldx, A, st); return true;
    case 512: launch_fwd<16>(p, B, x, ldx, A, st); return true;
    case 1024: launch_fwd<32>(p, B, x, ldx, A, st); return true;
    default: return false;
  }
}

bool xpass_warp_inv(const ConvPlan& p, int B, const float2* A, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                    const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st) {
  switch (p.X) {
    case 256: launch_inv<8>(p, B, A, x, ldx, y, ldy, scale, zdiag, zstride, st); return true;
    case 512: launch_inv<16>(p, B, A, x, ldx, y, ldy, scale, zdiag, zstride, st); return true;
    case 1024: launch_inv<32>(p, B, A, x, ldx, y, ldy, scale, zdiag, zstride, st); return true;
    default: return false;
  }
}

}  // namespace vh
