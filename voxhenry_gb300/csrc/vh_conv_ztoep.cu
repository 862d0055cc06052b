// Pass 3 of the complex64 and double-float FFT convolutions as a direct convolution along z (the
// autotuner's z_variant 3).  After the x- and y-transforms every (kx, ky) column holds nz voxel rows of the five
// current components, and the circulant's z-part acts on them as a Toeplitz operator: with the tensor
// spectrum S_k(kx, ky, kz) (already divided by X Y Z),
//   out[m] = sum_n h_k[m - n] in[n],   h_k[d] = sum_kz S_k[kz] e^{+2 pi i kz d / Z},   0 <= m, n < nz,
// which is exactly what the z-FFT, the product with S_k and the inverse z-FFT compute (the operator of
// lse_matvect_mult.m:57-93 along z).  For nz rows the direct form costs 13 nz^2 complex-by-real
// multiply-adds per column (13 distinct convolutions) against ten pruned Z-point transforms and 13 Z
// products, and needs no exchange between threads: at nz <= 16 it is the cheaper form.  The inputs
// of each right-hand side reach shared memory by tensor-memory-accelerator copies.
//
// The kernel is even or odd along each axis, so h_k is real (components 0, 3, 4, 5, 6) or imaginary
// (1, 2), even in d except for component 4 (odd): one float per (k, d >= 0).  The table is built on
// the device from the complex128 spectrum in FP64 and checked for that form (like the spectrum's own
// real/imaginary check); where it fails the variant is not offered.
#include <cuda.h>   // CUtensorMap (the encoder is looked up through the runtime)
#include <cudaTypedefs.h>

#include <cstddef>
#include <cstring>

#include "vh_conv.cuh"
#include "vh_df.cuh"

namespace vh {
namespace {

// h_k real (false) or imaginary (true), and its parity in d
__host__ __device__ constexpr bool zt_imag(int k) { return k == 1 || k == 2; }
__host__ __device__ constexpr int zt_parity(int k) { return k == 4 ? -1 : 1; }

// gz[((ky * 7 + k) * nz + d) * X + kx] for 0 <= d < nz (gzlo: the low float of the double-float pair
// whose high float is gz); mx[3k..3k+2]: max |kept part|, max |dropped
// part| and max |h_k[-d] - parity h_k[d]| as ordered bit patterns of non-negative doubles
__global__ void k_ztoep_table(const double2* __restrict__ tens, const double2* __restrict__ tw, int X, int Y, int Z,
                              int nz, float* __restrict__ gz, float* __restrict__ gzlo, unsigned long long* __restrict__ mx) {
  const int64_t n = (int64_t)X * Y * 7;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % X);
    const int k = (int)((idx / X) % 7);
    const int ky = (int)(idx / (7 * (int64_t)X));
    const double2* s = tens + ((int64_t)ky * Z * 7 + k) * X + kx;   // s[kz * 7 X]
    double keep_mx = 0.0, drop_mx = 0.0, par_mx = 0.0;
    for (int d = 0; d < nz; ++d) {
      double2 hp = make_double2(0.0, 0.0), hn = make_double2(0.0, 0.0);   // h[d], h[-d]
      for (int kz = 0; kz < Z; ++kz) {
        const double2 v = s[(int64_t)kz * 7 * X];
        const double2 w = tw[(int)(((int64_t)kz * d) % Z)];   // e^{-2 pi i kz d / Z}
        hp.x += v.x * w.x + v.y * w.y;   // v conj(w)
        hp.y += v.y * w.x - v.x * w.y;
        hn.x += v.x * w.x - v.y * w.y;   // v w
        hn.y += v.y * w.x + v.x * w.y;
      }
      const double keep = zt_imag(k) ? hp.y : hp.x;
      const double drop = zt_imag(k) ? hp.x : hp.y;
      const double keepn = zt_imag(k) ? hn.y : hn.x;
      const double dropn = zt_imag(k) ? hn.x : hn.y;
      const float hi = (float)keep;
      gz[(((int64_t)ky * 7 + k) * nz + d) * X + kx] = hi;
      gzlo[(((int64_t)ky * 7 + k) * nz + d) * X + kx] = (float)(keep - (double)hi);   // the pair's low part
      keep_mx = fmax(keep_mx, fabs(keep));
      drop_mx = fmax(drop_mx, fmax(fabs(drop), fabs(dropn)));
      par_mx = fmax(par_mx, fabs(keepn - zt_parity(k) * keep));
    }
    atomicMax(mx + 3 * k, (unsigned long long)__double_as_longlong(keep_mx));
    atomicMax(mx + 3 * k + 1, (unsigned long long)__double_as_longlong(drop_mx));
    atomicMax(mx + 3 * k + 2, (unsigned long long)__double_as_longlong(par_mx));
  }
}

constexpr int kZtCols = 32;

// shared-memory row stride of a column's h values: a multiple of 4 floats with an odd number of
// 16-byte chunks, so that the 8 lanes of a quarter-warp's 16-byte loads hit 8 different bank quads
__host__ __device__ constexpr int zt_gstride(int nz) { return ((nz + 3) / 4) % 2 ? (nz + 3) / 4 * 4 : (nz + 3) / 4 * 4 + 4; }

// One convolution step into acc: acc[m] += sum_n h[m - n] v(n), h[d] = g[d] for d >= 0 and
// h[-d] = (ODD ? -1 : 1) g[d]; v(n) = p1[n] or, PAIR, i (p1[n] + s2 p2[n]) (the two combined inputs
// of the operator are both taken times an imaginary kernel); p1[n] is row n of a staged component
// (rows nz .. NZ - 1 are zero).  A fully unrolled body: the kernel instantiates three of them and
// every warp runs its steps through these three, so the hot code stays small.
template <int NZ, bool ODD, bool PAIR>
__device__ __forceinline__ void zt_conv(float2 (&acc)[NZ], const float* grow, const float2* p1, const float2* p2,
                                        float s2) {
  float g[NZ];
#pragma unroll
  for (int d = 0; d < NZ; d += 4) {
    const float4 q = *reinterpret_cast<const float4*>(grow + d);
    g[d] = q.x;
    if (d + 1 < NZ) g[d + 1] = q.y;
    if (d + 2 < NZ) g[d + 2] = q.z;
    if (d + 3 < NZ) g[d + 3] = q.w;
  }
#pragma unroll
  for (int n = 0; n < NZ; ++n) {
    float2 v = p1[n * kZtCols];
    if (PAIR) {
      const float2 u = p2[n * kZtCols];
      v.x = fmaf(s2, u.x, v.x);   // = v + s2 u with s2 = +-1, rounded once
      v.y = fmaf(s2, u.y, v.y);
    }
#pragma unroll
    for (int m = 0; m < NZ; ++m) {
      const int d = m - n;
      const float w = g[d >= 0 ? d : -d];
      const float ws = (d < 0 && ODD) ? -w : w;
      if (PAIR) {
        acc[m].x = fmaf(-ws, v.y, acc[m].x);
        acc[m].y = fmaf(ws, v.x, acc[m].y);
      } else {
        acc[m].x = fmaf(ws, v.x, acc[m].x);
        acc[m].y = fmaf(ws, v.y, acc[m].y);
      }
    }
  }
}

// ---- staging by the tensor memory accelerator.  The right-hand sides' five components are one 3-D
// tensor of 64-bit elements: x = kx (W elements per value: 1 for complex64, 2 for the double-float
// pairs), y = ky, z = the row (b * 5 + c) * nz + n.  One copy moves a box of 32 columns x 1 x nz rows
// (one component of one RHS) into in[c][0 .. nz); columns past the grid's last read as zeros.  Its
// x coordinate is a multiple of 32 W elements (256 W bytes), the 16-byte rule of tiled copies.
constexpr unsigned kZtWaitLimit = 1u << 20;   // polls of an mbarrier before the pass gives up

__device__ __forceinline__ unsigned zt_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void zt_mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(zt_smem(bar)) : "memory");
}
// the initialised barriers visible to the copy engine and to every thread (after a __syncthreads)
__device__ __forceinline__ void zt_mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}
// the threads' earlier shared-memory accesses ordered before the copies issued next
__device__ __forceinline__ void zt_fence_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void zt_mbar_expect(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(zt_smem(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void zt_tma_load(const CUtensorMap* map, void* dst, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(zt_smem(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(zt_smem(bar))
      : "memory");
}

// waits for the phase of `parity` to complete; false after kZtWaitLimit polls
__device__ __forceinline__ bool zt_mbar_wait(uint64_t* bar, unsigned parity) {
  for (unsigned i = 0; i < kZtWaitLimit; ++i) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(zt_smem(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// set when a pass gave up waiting for its copies (its outputs are then NaN)
__device__ int g_zt_stalled;

// thread 0: the five components of RHS b into in[0..4] (component stride `cstride` bytes), completing
// on `bar`
__device__ __forceinline__ void zt_issue(const CUtensorMap* map, unsigned char* in0, size_t cstride, uint64_t* bar,
                                         int x, int ky, int b, int nz, unsigned bytes) {
  zt_fence_async();
  zt_mbar_expect(bar, bytes);
#pragma unroll 1
  for (int c = 0; c < 5; ++c) zt_tma_load(map, in0 + c * cstride, bar, x, ky, (b * 5 + c) * nz);
}

__device__ __forceinline__ void zt_bar_arrive() { asm volatile("bar.arrive 1, 160;\n" ::: "memory"); }
__device__ __forceinline__ void zt_bar_sync() { asm volatile("bar.sync 1, 160;\n" ::: "memory"); }

// Five warps over 32 columns of one ky row (lane = column), all right-hand sides of the batch; the
// 13 distinct convolutions of the operator (tensor_apply_ri in the spectral form) split 3/3/3/2/2:
//   warp 0: A = G1 jx,  then o0 = G0 jx + G1 (j2 + j3)
//   warp 1: B = G2 jy,  then o1 = G0 jy + G2 (j2 - j3)
//   warp 2: P = G4 jz,  then o2 = G0 jz + G4 j3
//   warp 3: o3 = G3 j2 + G5 j3 - A - B
//   warp 4: o4 = G5 j2 + G6 j3 - A + B - P
// A, B and P are computed first and pass through shared memory (named barrier 1: warps 0-2 arrive,
// 3-4 wait), so that warps 3-4 rarely wait for them.  G1 and G2 are imaginary: their combined inputs
// run through the PAIR body; A and B run through the real body and are rotated by i when stored.
// Each RHS's inputs are staged in shared memory (double-buffered: the next RHS's copies are in flight
// while this one is computed; rows nz .. NZ - 1 stay zero), so the in-place stores never meet another
// warp's loads.
//
// A step is coded as kind (bits 0-1: 0 even kernel, 1 combined inputs, 2 odd kernel), kernel k (bits
// 2-4), first input (5-7), second input (8-10), second input subtracted (bit 11).
__constant__ unsigned short kZtProgram[5][3] = {
    {0 | 1 << 2 | 0 << 5, 0 | 0 << 2 | 0 << 5, 1 | 1 << 2 | 3 << 5 | 4 << 8},
    {0 | 2 << 2 | 1 << 5, 0 | 0 << 2 | 1 << 5, 1 | 2 << 2 | 3 << 5 | 4 << 8 | 1 << 11},
    {2 | 4 << 2 | 2 << 5, 0 | 0 << 2 | 2 << 5, 2 | 4 << 2 | 4 << 5},
    {0, 0 | 3 << 2 | 3 << 5, 0 | 5 << 2 | 4 << 5},
    {0, 0 | 5 << 2 | 3 << 5, 0 | 6 << 2 | 4 << 5}};

template <int NZ>
struct ZtSmem {
  static constexpr int GST = zt_gstride(NZ);
  float g[7][kZtCols][GST];               // h_k of each column, rows d >= nz zero
  float2 in[2][5][NZ][kZtCols];           // staged RHS (double-buffered), 128-byte aligned
  float2 part[3][NZ][kZtCols];            // A, B, P for the last two warps
  uint64_t bar[2];                        // completion of each buffer's copies
};

template <int NZ>
__global__ void __launch_bounds__(5 * 32) k_zpass_toep(const __grid_constant__ CUtensorMap map, float2* __restrict__ Bf,
                                                      const float* __restrict__ gz, int nz, int Y, int X, int nrhs) {
  static_assert(offsetof(ZtSmem<NZ>, in) % 128 == 0, "copy destinations 128-byte aligned");
  extern __shared__ __align__(128) unsigned char zt_raw[];
  ZtSmem<NZ>& sm = *reinterpret_cast<ZtSmem<NZ>*>(zt_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ky = blockIdx.y;
  const int kx0 = blockIdx.x * kZtCols;
  const int kx = kx0 + lane;
  const bool ok = kx < X;
  const int64_t plane = (int64_t)Y * X;       // one z row of one component
  const int64_t comp = (int64_t)nz * plane;   // one component of one RHS
  constexpr size_t cbytes = sizeof(sm.in[0][0]);                       // one staged component
  const unsigned bytes = 5u * (unsigned)nz * kZtCols * sizeof(float2);   // one RHS's copies
  for (int i = threadIdx.x; i < 2 * 5 * NZ * kZtCols; i += blockDim.x) {   // padding rows nz.. stay zero
    const int cc = i % kZtCols, n = (i / kZtCols) % NZ, cb = i / (kZtCols * NZ);
    if (n >= nz) sm.in[cb / 5][cb % 5][n][cc] = make_float2(0.0f, 0.0f);
  }
  if (threadIdx.x == 0) {
    zt_mbar_init(&sm.bar[0]);
    zt_mbar_init(&sm.bar[1]);
    zt_mbar_fence_init();
  }
  __syncthreads();
  // the copies want 128-byte aligned destinations (checked, not assumed: a pass that cannot copy says so)
  const bool aligned = (zt_smem(sm.in) & 127u) == 0;
  int last = -1;   // thread 0: the last RHS whose copies it issued
  if (threadIdx.x == 0 && nrhs > 0 && aligned) {
    zt_issue(&map, reinterpret_cast<unsigned char*>(sm.in[0]), cbytes, &sm.bar[0], kx0, ky, 0, nz, bytes);
    last = 0;
  }
  for (int i = threadIdx.x; i < 7 * NZ * kZtCols; i += blockDim.x) {
    const int cc = i % kZtCols, d = (i / kZtCols) % NZ, k = i / (kZtCols * NZ);
    sm.g[k][cc][d] = (kx0 + cc < X && d < nz) ? gz[(((int64_t)ky * 7 + k) * nz + d) * X + kx0 + cc] : 0.0f;
  }
  const float* gl = &sm.g[0][lane][0];
  constexpr int gk = kZtCols * ZtSmem<NZ>::GST;   // g[k + 1] - g[k]
  constexpr int ck = NZ * kZtCols;                // in[c + 1] - in[c]
  bool stalled = !aligned;
  for (int b = 0; b < nrhs; ++b) {
    if (!stalled) stalled = !zt_mbar_wait(&sm.bar[b & 1], (b >> 1) & 1);   // RHS b staged
    // every warp is done with RHS b - 1 (its buffer and the partial sums)
    __syncthreads();
    if (threadIdx.x == 0 && b + 1 < nrhs && !stalled) {
      zt_issue(&map, reinterpret_cast<unsigned char*>(sm.in[(b + 1) & 1]), cbytes, &sm.bar[(b + 1) & 1], kx0, ky,
               b + 1, nz, bytes);
      last = b + 1;
    }
    const float2* s = &sm.in[b & 1][0][0][lane];
    float2 acc[NZ];
#pragma unroll
    for (int m = 0; m < NZ; ++m) acc[m] = make_float2(0.0f, 0.0f);
#pragma unroll 1
    for (int st = warp < 3 ? 0 : 1; st < 3; ++st) {
      const unsigned code = kZtProgram[warp][st];
      const float* gr = gl + ((code >> 2) & 7) * gk;
      const float2* p1 = s + ((code >> 5) & 7) * ck;
      switch (code & 3) {
        case 0: zt_conv<NZ, false, false>(acc, gr, p1, p1, 0.0f); break;
        case 1: zt_conv<NZ, false, true>(acc, gr, p1, s + ((code >> 8) & 7) * ck, (code >> 11) & 1 ? -1.0f : 1.0f); break;
        default: zt_conv<NZ, true, false>(acc, gr, p1, p1, 0.0f); break;
      }
      if (st == 0) {   // A, B (times i: G1 and G2 are imaginary) or P for warps 3-4; acc starts over
        const bool rot = warp < 2;
#pragma unroll
        for (int m = 0; m < NZ; ++m) {
          sm.part[warp][m][lane] = rot ? make_float2(-acc[m].y, acc[m].x) : acc[m];
          acc[m] = make_float2(0.0f, 0.0f);
        }
        zt_bar_arrive();
      }
    }
    if (warp == 3) {
      zt_bar_sync();
#pragma unroll
      for (int m = 0; m < NZ; ++m) {
        const float2 a = sm.part[0][m][lane], bb = sm.part[1][m][lane];
        acc[m].x -= a.x + bb.x;
        acc[m].y -= a.y + bb.y;
      }
    } else if (warp == 4) {
      zt_bar_sync();
#pragma unroll
      for (int m = 0; m < NZ; ++m) {
        const float2 a = sm.part[0][m][lane], bb = sm.part[1][m][lane], pp = sm.part[2][m][lane];
        acc[m].x += (bb.x - a.x) - pp.x;
        acc[m].y += (bb.y - a.y) - pp.y;
      }
    }
    if (stalled) {   // the copies never completed: the product is NaN, and the pass says so
#pragma unroll
      for (int m = 0; m < NZ; ++m) acc[m] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
      g_zt_stalled = 1;
    }
    if (ok) {   // the warp's output component
      float2* out = Bf + (int64_t)b * 5 * comp + (int64_t)warp * comp + (int64_t)ky * X + kx;
#pragma unroll
      for (int m = 0; m < NZ; ++m)
        if (m < nz) out[m * plane] = acc[m];
    }
  }
  // thread 0 issues only after its own wait succeeded, so when it gave up, the copies it waited for
  // (its last issue) may still be in flight: one more bounded wait before the block's shared memory
  // is released
  if (threadIdx.x == 0 && stalled && last >= 0) zt_mbar_wait(&sm.bar[last & 1], (last >> 1) & 1);
}

// ---- the same pass in double-float arithmetic (VH_PREC_DF: pair storage of Bf, pair h values, each
// output a Dot2 accumulation over all its terms, ~48 significant bits); single-buffered staging.
// A pair multiply-add is about twelve instructions, so a fully unrolled convolution would be several
// kilobytes of code per step: the body loops over the input rows at run time, reads the row's NZ
// kernel values from a two-sided table in shared memory (h2[k][j] = h_k[j - (NZ - 1)], the parity
// already applied) and serves every step of every warp.
template <int NZ>
struct ZtSmemDf {
  dfloat h2[7][2 * NZ - 1][kZtCols];
  dcomplex in[5][NZ][kZtCols];   // 128-byte aligned
  dcomplex part[3][NZ][kZtCols];
  uint64_t bar;
};

// (re, im)[m] += sum_n h[m - n] v(n) for n < nz; v(n) = p1[n] (+ or - p2[n] with PAIR), times i with
// IMAG; H = &h2[k][0][lane]
template <int NZ>
__device__ __forceinline__ void zt_conv_df(df_dot (&re)[NZ], df_dot (&im)[NZ], const dfloat* H, const dcomplex* p1,
                                           const dcomplex* p2, int nz, bool pair, bool neg2, bool imag) {
#pragma unroll 1
  for (int n = 0; n < nz; ++n) {
    dcomplex v = p1[n * kZtCols];
    if (pair) {
      const dcomplex u = p2[n * kZtCols];
      v = neg2 ? dcomplex{v.x - u.x, v.y - u.y} : dcomplex{v.x + u.x, v.y + u.y};
    }
    const dfloat vx = imag ? -v.y : v.x, vy = imag ? v.x : v.y;
    const dfloat* w = H + (NZ - 1 - n) * kZtCols;   // w[m * kZtCols] = h[m - n]
#pragma unroll
    for (int m = 0; m < NZ; ++m) {
      const dfloat wm = w[m * kZtCols];
      re[m].add(wm, vx);
      im[m].add(wm, vy);
    }
  }
}

template <int NZ>
__global__ void __launch_bounds__(5 * 32) k_zpass_toep_df(const __grid_constant__ CUtensorMap map,
                                                         dcomplex* __restrict__ Bf, const float* __restrict__ gz,
                                                         const float* __restrict__ gzlo, int nz, int Y, int X,
                                                         int nrhs) {
  static_assert(offsetof(ZtSmemDf<NZ>, in) % 128 == 0, "copy destinations 128-byte aligned");
  extern __shared__ __align__(128) unsigned char zt_raw[];
  ZtSmemDf<NZ>& sm = *reinterpret_cast<ZtSmemDf<NZ>*>(zt_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ky = blockIdx.y;
  const int kx0 = blockIdx.x * kZtCols;
  const int kx = kx0 + lane;
  const bool ok = kx < X;
  const int64_t plane = (int64_t)Y * X;
  const int64_t comp = (int64_t)nz * plane;
  for (int i = threadIdx.x; i < 5 * NZ * kZtCols; i += blockDim.x) {   // padding rows nz.. stay zero
    const int col = i % kZtCols, n = (i / kZtCols) % NZ, c = i / (kZtCols * NZ);
    if (n >= nz) sm.in[c][n][col] = dcomplex{dfloat(0.0f), dfloat(0.0f)};
  }
  if (threadIdx.x == 0) {
    zt_mbar_init(&sm.bar);
    zt_mbar_fence_init();
  }
  for (int i = threadIdx.x; i < 7 * (2 * NZ - 1) * kZtCols; i += blockDim.x) {
    const int col = i % kZtCols, j = (i / kZtCols) % (2 * NZ - 1), k = i / (kZtCols * (2 * NZ - 1));
    const int d = j - (NZ - 1), ad = d < 0 ? -d : d;
    dfloat h(0.0f);
    if (kx0 + col < X && ad < nz) {
      const int64_t gi = (((int64_t)ky * 7 + k) * nz + ad) * X + kx0 + col;
      h = dfloat(gz[gi], gzlo[gi]);
      if (d < 0 && zt_parity(k) < 0) h = -h;
    }
    sm.h2[k][j][col] = h;
  }
  constexpr int ck = NZ * kZtCols;   // in[c + 1] - in[c]
  const unsigned bytes = 5u * (unsigned)nz * kZtCols * sizeof(dcomplex);
  bool stalled = (zt_smem(sm.in) & 127u) != 0;   // the copies want 128-byte aligned destinations
  int last = -1;                                  // thread 0: the last RHS whose copies it issued
  for (int b = 0; b < nrhs; ++b) {
    // every warp is done with RHS b - 1 (the staged inputs and the partial sums); the barrier is
    // initialised and the table written (first pass)
    __syncthreads();
    if (threadIdx.x == 0 && !stalled) {
      zt_issue(&map, reinterpret_cast<unsigned char*>(sm.in), sizeof(sm.in[0]), &sm.bar, 2 * kx0, ky, b, nz, bytes);
      last = b;
    }
    if (!stalled) stalled = !zt_mbar_wait(&sm.bar, b & 1);
    const dcomplex* s = &sm.in[0][0][lane];
    df_dot re[NZ], im[NZ];
#pragma unroll
    for (int m = 0; m < NZ; ++m) re[m] = im[m] = df_dot(dfloat(0.0f));
#pragma unroll 1
    for (int st = warp < 3 ? 0 : 1; st < 3; ++st) {   // the warp's steps, as in k_zpass_toep
      const unsigned code = kZtProgram[warp][st];
      const int k = (code >> 2) & 7;
      zt_conv_df<NZ>(re, im, &sm.h2[k][0][lane], s + ((code >> 5) & 7) * ck, s + ((code >> 8) & 7) * ck, nz,
                     (code & 3) == 1, (code >> 11) & 1, zt_imag(k));
      if (st == 0) {   // A, B or P for warps 3-4; the accumulators start over
#pragma unroll
        for (int m = 0; m < NZ; ++m) {
          sm.part[warp][m][lane] = dcomplex{re[m].value(), im[m].value()};
          re[m] = im[m] = df_dot(dfloat(0.0f));
        }
        zt_bar_arrive();
      }
    }
    if (warp == 3) {
      zt_bar_sync();
#pragma unroll
      for (int m = 0; m < NZ; ++m) {
        const dcomplex a = sm.part[0][m][lane], bb = sm.part[1][m][lane];
        re[m].merge(-a.x.hi, -a.x.lo);
        re[m].merge(-bb.x.hi, -bb.x.lo);
        im[m].merge(-a.y.hi, -a.y.lo);
        im[m].merge(-bb.y.hi, -bb.y.lo);
      }
    } else if (warp == 4) {
      zt_bar_sync();
#pragma unroll
      for (int m = 0; m < NZ; ++m) {
        const dcomplex a = sm.part[0][m][lane], bb = sm.part[1][m][lane], pp = sm.part[2][m][lane];
        re[m].merge(-a.x.hi, -a.x.lo);
        re[m].merge(bb.x.hi, bb.x.lo);
        re[m].merge(-pp.x.hi, -pp.x.lo);
        im[m].merge(-a.y.hi, -a.y.lo);
        im[m].merge(bb.y.hi, bb.y.lo);
        im[m].merge(-pp.y.hi, -pp.y.lo);
      }
    }
    if (stalled) {   // the copies never completed: the product is NaN, and the pass says so
      const float qnan = __int_as_float(0x7fc00000);
#pragma unroll
      for (int m = 0; m < NZ; ++m) re[m] = im[m] = df_dot(dfloat(qnan));
      g_zt_stalled = 1;
    }
    if (ok) {   // the warp's output component
      dcomplex* out = Bf + (int64_t)b * 5 * comp + (int64_t)warp * comp + (int64_t)ky * X + kx;
#pragma unroll
      for (int m = 0; m < NZ; ++m)
        if (m < nz) out[m * plane] = dcomplex{re[m].value(), im[m].value()};
    }
  }
  // a copy thread 0 gave up on may still be in flight: one more bounded wait before exit
  if (threadIdx.x == 0 && stalled && last >= 0) zt_mbar_wait(&sm.bar, last & 1);
}

// the driver's tensor-map encoder, looked up once through the runtime
PFN_cuTensorMapEncodeTiled_v12000 zt_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    cudaGetLastError();
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// The staging tensor of the B right-hand sides in Bf (W 64-bit elements per value); false where the
// layout does not meet the copy engine's rules (16-byte base and row strides), and the pass is then not
// run (the FFT z-pass runs instead).
bool zt_tensor_map(CUtensorMap* map, const void* Bf, int W, int X, int Y, int B, int nz) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = zt_encoder();
  const uint64_t row = (uint64_t)X * W * 8;
  if (!enc || reinterpret_cast<uintptr_t>(Bf) % 16 != 0 || row % 16 != 0) return false;
  const cuuint64_t dim[3] = {(cuuint64_t)X * W, (cuuint64_t)Y, (cuuint64_t)B * 5 * nz};
  const cuuint64_t stride[2] = {row, row * (uint64_t)Y};
  const cuuint32_t box[3] = {(cuuint32_t)(kZtCols * W), 1u, (cuuint32_t)nz};
  const cuuint32_t step[3] = {1u, 1u, 1u};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void*>(Bf), dim, stride, box, step,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NZ>
bool launch_zpass_toep_df(dcomplex* Bf, const float* gz, const float* gzlo, int nz, int Y, int X, int B,
                          cudaStream_t st) {
  CUtensorMap map;
  if (!zt_tensor_map(&map, Bf, 2, X, Y, B, nz)) return false;
  constexpr size_t sm = sizeof(ZtSmemDf<NZ>);
  allow_dyn_smem(k_zpass_toep_df<NZ>, sm);
  dim3 grid((unsigned)ceil_div(X, kZtCols), (unsigned)Y);
  k_zpass_toep_df<NZ><<<grid, 5 * 32, sm, st>>>(map, Bf, gz, gzlo, nz, Y, X, B);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  return true;
}

template <int NZ>
bool launch_zpass_toep(float2* Bf, const float* gz, int nz, int Y, int X, int B, cudaStream_t st) {
  CUtensorMap map;
  if (!zt_tensor_map(&map, Bf, 1, X, Y, B, nz)) return false;
  constexpr size_t sm = sizeof(ZtSmem<NZ>);
  allow_dyn_smem(k_zpass_toep<NZ>, sm);
  dim3 grid((unsigned)ceil_div(X, kZtCols), (unsigned)Y);
  k_zpass_toep<NZ><<<grid, 5 * 32, sm, st>>>(map, Bf, gz, nz, Y, X, B);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  return true;
}

}  // namespace

bool ztoep_build(ConvPlan& p, cudaStream_t st) {
  if (p.ztoep_state != 0) return p.ztoep_state > 0;
  p.ztoep_state = -1;
  if (p.nz < 1 || p.nz > kZtoepMaxRows || !p.tens64 || !p.tw64[2]) return false;
  const int64_t n = (int64_t)7 * p.nz * p.Y * p.X;
  float* gz = nullptr;
  unsigned long long* d_mx = nullptr;
  VH_CUDA_TRY(cudaMalloc(&gz, 2 * n * sizeof(float)));   // high floats, then the pairs' low floats
  try {
    VH_CUDA_TRY(cudaMalloc(&d_mx, 21 * sizeof(unsigned long long)));
    VH_CUDA_TRY(cudaMemsetAsync(d_mx, 0, 21 * sizeof(unsigned long long), st));
    k_ztoep_table<<<2048, 256, 0, st>>>(p.tens64, p.tw64[2], p.X, p.Y, p.Z, p.nz, gz, gz + n, d_mx);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    unsigned long long hmx[21];
    VH_CUDA_TRY(cudaMemcpyAsync(hmx, d_mx, sizeof(hmx), cudaMemcpyDeviceToHost, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFree(d_mx);
    d_mx = nullptr;
    bool ok = true;
    for (int k = 0; k < 7; ++k) {
      double v[3];
      std::memcpy(v, hmx + 3 * k, sizeof(v));
      ok = ok && v[1] <= 1e-9 * v[0] && v[2] <= 1e-9 * v[0];
    }
    if (!ok) {
      cudaFree(gz);
      return false;
    }
  } catch (...) {
    cudaFree(d_mx);
    cudaFree(gz);
    throw;
  }
  p.tensz = gz;
  p.ztoep_state = 1;
  return true;
}

bool ztoep_take_stall(cudaStream_t st) {
  int v = 0;
  VH_CUDA_TRY(cudaMemcpyFromSymbolAsync(&v, g_zt_stalled, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  VH_CUDA_TRY(cudaStreamSynchronize(st));
  if (v != 0) {
    const int zero = 0;
    VH_CUDA_TRY(cudaMemcpyToSymbolAsync(g_zt_stalled, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return v != 0;
}

bool zpass_toep_df(const ConvPlan& p, dcomplex* Bf, int B, cudaStream_t st) {
  if (p.ztoep_state <= 0 || !p.tensz) return false;
  const int nz = p.nz;
  const float* lo = p.tensz + (int64_t)7 * nz * p.Y * p.X;
  switch ((nz + 1) / 2) {
    case 1: return launch_zpass_toep_df<2>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 2: return launch_zpass_toep_df<4>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 3: return launch_zpass_toep_df<6>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 4: return launch_zpass_toep_df<8>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 5: return launch_zpass_toep_df<10>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 6: return launch_zpass_toep_df<12>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 7: return launch_zpass_toep_df<14>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    case 8: return launch_zpass_toep_df<16>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st);
    default: return false;
  }
}

bool zpass_toep(const ConvPlan& p, float2* Bf, int B, cudaStream_t st) {
  if (p.ztoep_state <= 0 || !p.tensz) return false;
  const int nz = p.nz;
  switch ((nz + 1) / 2) {
    case 1: return launch_zpass_toep<2>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 2: return launch_zpass_toep<4>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 3: return launch_zpass_toep<6>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 4: return launch_zpass_toep<8>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 5: return launch_zpass_toep<10>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 6: return launch_zpass_toep<12>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 7: return launch_zpass_toep<14>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    case 8: return launch_zpass_toep<16>(Bf, p.tensz, nz, p.Y, p.X, B, st);
    default: return false;
  }
}

}  // namespace vh
