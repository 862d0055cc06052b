// Pass 3 of the complex64 FFT convolution as a direct convolution along z (the autotuner's
// z_variant 3).  After the x- and y-transforms every (kx, ky) column holds nz voxel rows of the five
// current components, and the circulant's z-part acts on them as a Toeplitz operator: with the tensor
// spectrum S_k(kx, ky, kz) (already divided by X Y Z),
//   out[m] = sum_n h_k[m - n] in[n],   h_k[d] = sum_kz S_k[kz] e^{+2 pi i kz d / Z},   0 <= m, n < nz,
// which is exactly what the z-FFT, the product with S_k and the inverse z-FFT compute (the operator of
// lse_matvect_mult.m:57-93 along z).  For nz rows the direct form costs 15 nz^2 complex-by-real
// multiply-adds per column against ten pruned Z-point transforms and 13 Z products, and needs no
// exchange between threads: at nz <= 16 it is the cheaper form.
//
// The kernel is even or odd along each axis, so h_k is real (components 0, 3, 4, 5, 6) or imaginary
// (1, 2), even in d except for component 4 (odd): one float per (k, d >= 0).  The table is built on
// the device from the complex128 spectrum in FP64 and checked for that form (like the spectrum's own
// real/imaginary check); where it fails the variant is not offered.
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

__device__ __forceinline__ void zt_cp16(void* dst, const void* src) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void zt_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void zt_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Stages RHS b's five components (nz rows x 32 columns) into in[c][n][32] with 16-byte cp.async
// copies (two columns each), thread t taking rows t/16, t/16 + 10, ... at column pair t % 16;
// copies past the grid's last column are skipped.
template <int NZ>
__device__ __forceinline__ void zt_stage(float2 (*dst)[NZ][kZtCols], const float2* src, int nz, int64_t plane,
                                         int64_t comp, int kx0, int X) {
  const int q = threadIdx.x % (kZtCols / 2);
  const bool ok = kx0 + 2 * q < X;
  int c = 0, n = threadIdx.x / (kZtCols / 2);   // row c * nz + n, advanced by 10 rows per copy
  while (n >= nz) { n -= nz; ++c; }
  for (; c < 5;) {
    if (ok) zt_cp16(&dst[c][n][2 * q], src + c * comp + n * plane + 2 * q);
    n += (5 * kZtCols) / (kZtCols / 2);
    while (n >= nz && c < 5) { n -= nz; ++c; }
  }
  zt_commit();
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
  float2 in[2][5][NZ][kZtCols];           // staged RHS (double-buffered)
  float2 part[3][NZ][kZtCols];            // A, B, P for the last two warps
};

template <int NZ>
__global__ void __launch_bounds__(5 * 32) k_zpass_toep(float2* __restrict__ Bf, const float* __restrict__ gz, int nz,
                                                      int Y, int X, int nrhs) {
  extern __shared__ __align__(16) unsigned char zt_raw[];
  ZtSmem<NZ>& sm = *reinterpret_cast<ZtSmem<NZ>*>(zt_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ky = blockIdx.y;
  const int kx0 = blockIdx.x * kZtCols;
  const int kx = kx0 + lane;
  const bool ok = kx < X;
  const int64_t plane = (int64_t)Y * X;       // one z row of one component
  const int64_t comp = (int64_t)nz * plane;   // one component of one RHS
  const float2* src0 = Bf + (int64_t)ky * X + kx0;
  for (int i = threadIdx.x; i < 2 * 5 * NZ * kZtCols; i += blockDim.x) {   // padding rows nz.. stay zero
    const int cc = i % kZtCols, n = (i / kZtCols) % NZ, cb = i / (kZtCols * NZ);
    if (n >= nz) sm.in[cb / 5][cb % 5][n][cc] = make_float2(0.0f, 0.0f);
  }
  if (nrhs > 0) zt_stage<NZ>(sm.in[0], src0, nz, plane, comp, kx0, X);
  for (int i = threadIdx.x; i < 7 * NZ * kZtCols; i += blockDim.x) {
    const int cc = i % kZtCols, d = (i / kZtCols) % NZ, k = i / (kZtCols * NZ);
    sm.g[k][cc][d] = (kx0 + cc < X && d < nz) ? gz[(((int64_t)ky * 7 + k) * nz + d) * X + kx0 + cc] : 0.0f;
  }
  const float* gl = &sm.g[0][lane][0];
  constexpr int gk = kZtCols * ZtSmem<NZ>::GST;   // g[k + 1] - g[k]
  constexpr int ck = NZ * kZtCols;                // in[c + 1] - in[c]
  for (int b = 0; b < nrhs; ++b) {
    zt_wait<0>();
    // RHS b staged by every thread; every warp is done with RHS b - 1 (its buffer and the partial sums)
    __syncthreads();
    if (b + 1 < nrhs) zt_stage<NZ>(sm.in[(b + 1) & 1], src0 + (int64_t)(b + 1) * 5 * comp, nz, plane, comp, kx0, X);
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
    if (ok) {   // the warp's output component
      float2* out = Bf + (int64_t)b * 5 * comp + (int64_t)warp * comp + (int64_t)ky * X + kx;
#pragma unroll
      for (int m = 0; m < NZ; ++m)
        if (m < nz) out[m * plane] = acc[m];
    }
  }
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
  dcomplex in[5][NZ][kZtCols];
  dcomplex part[3][NZ][kZtCols];
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
__global__ void __launch_bounds__(5 * 32) k_zpass_toep_df(dcomplex* __restrict__ Bf, const float* __restrict__ gz,
                                                         const float* __restrict__ gzlo, int nz, int Y, int X,
                                                         int nrhs) {
  extern __shared__ __align__(16) unsigned char zt_raw[];
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
  for (int b = 0; b < nrhs; ++b) {
    __syncthreads();   // every warp is done with RHS b - 1 (the staged inputs and the partial sums)
    {
      const dcomplex* src = Bf + (int64_t)b * 5 * comp + (int64_t)ky * X + kx0;
      for (int i = threadIdx.x; i < 5 * nz * kZtCols; i += blockDim.x) {   // one 16-byte value per copy
        const int col = i % kZtCols, cn = i / kZtCols;
        const int c = cn / nz, n = cn - c * nz;
        if (kx0 + col < X) zt_cp16(&sm.in[c][n][col], src + c * comp + n * plane + col);
      }
      zt_commit();
      zt_wait<0>();
    }
    __syncthreads();
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
    if (ok) {   // the warp's output component
      dcomplex* out = Bf + (int64_t)b * 5 * comp + (int64_t)warp * comp + (int64_t)ky * X + kx;
#pragma unroll
      for (int m = 0; m < NZ; ++m)
        if (m < nz) out[m * plane] = dcomplex{re[m].value(), im[m].value()};
    }
  }
}

template <int NZ>
void launch_zpass_toep_df(dcomplex* Bf, const float* gz, const float* gzlo, int nz, int Y, int X, int B,
                          cudaStream_t st) {
  constexpr size_t sm = sizeof(ZtSmemDf<NZ>);
  allow_dyn_smem(k_zpass_toep_df<NZ>, sm);
  dim3 grid((unsigned)ceil_div(X, kZtCols), (unsigned)Y);
  k_zpass_toep_df<NZ><<<grid, 5 * 32, sm, st>>>(Bf, gz, gzlo, nz, Y, X, B);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

template <int NZ>
void launch_zpass_toep(float2* Bf, const float* gz, int nz, int Y, int X, int B, cudaStream_t st) {
  constexpr size_t sm = sizeof(ZtSmem<NZ>);
  allow_dyn_smem(k_zpass_toep<NZ>, sm);
  dim3 grid((unsigned)ceil_div(X, kZtCols), (unsigned)Y);
  k_zpass_toep<NZ><<<grid, 5 * 32, sm, st>>>(Bf, gz, nz, Y, X, B);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
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

bool zpass_toep_df(const ConvPlan& p, dcomplex* Bf, int B, cudaStream_t st) {
  if (p.ztoep_state <= 0 || !p.tensz) return false;
  const int nz = p.nz;
  const float* lo = p.tensz + (int64_t)7 * nz * p.Y * p.X;
  switch ((nz + 1) / 2) {
    case 1: launch_zpass_toep_df<2>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 2: launch_zpass_toep_df<4>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 3: launch_zpass_toep_df<6>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 4: launch_zpass_toep_df<8>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 5: launch_zpass_toep_df<10>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 6: launch_zpass_toep_df<12>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 7: launch_zpass_toep_df<14>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    case 8: launch_zpass_toep_df<16>(Bf, p.tensz, lo, nz, p.Y, p.X, B, st); break;
    default: return false;
  }
  return true;
}

bool zpass_toep(const ConvPlan& p, float2* Bf, int B, cudaStream_t st) {
  if (p.ztoep_state <= 0 || !p.tensz) return false;
  const int nz = p.nz;
  switch ((nz + 1) / 2) {
    case 1: launch_zpass_toep<2>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 2: launch_zpass_toep<4>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 3: launch_zpass_toep<6>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 4: launch_zpass_toep<8>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 5: launch_zpass_toep<10>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 6: launch_zpass_toep<12>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 7: launch_zpass_toep<14>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    case 8: launch_zpass_toep<16>(Bf, p.tensz, nz, p.Y, p.X, B, st); break;
    default: return false;
  }
  return true;
}

}  // namespace vh
