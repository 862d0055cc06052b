// Passes of the FFT convolution (the algorithm is described at the top of vh_conv.cu): the pass
// kernels, their launch shapes and conv_apply_t, templated on the arithmetic type -- float
// (complex64), double (complex128) and dfloat (double-float pairs).  Each type is instantiated in its
// own translation unit (vh_conv.cu, vh_conv_c64.cu, vh_conv_df.cu) so that the three compile in
// parallel.
#pragma once
#include <algorithm>
#include <type_traits>

#include "vh_conv.cuh"
#include "vh_df.cuh"

namespace vh {

// ------------------------------------------------------------------------------------------
template <typename T> struct TileCfg;
template <> struct TileCfg<double> { static constexpr int target = 2048; };
template <> struct TileCfg<float> { static constexpr int target = 2048; };
template <> struct TileCfg<dfloat> { static constexpr int target = 2048; };

static int x_lines_per_cta(int X, int target) { return std::max(1, std::min(64, target / X)); }
// columns per y-pass tile: even (16-byte chunks of complex64), smem ping-pong buffers <= ~72 KB
static int y_lines_per_cta(int Y, int X, bool dbl) {
  int tx = dbl ? 4 : 8;
  while (tx > 2 && (int64_t)2 * Y * tx * (dbl ? 16 : 8) > 72 * 1024) tx /= 2;
  return std::max(dbl ? 1 : 2, std::min(tx, X));
}

// ---- asynchronous 16-byte global -> shared copies (many in flight per thread)
__device__ __forceinline__ void cp_async16(void* s, const void* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// rows x cols tile from global (row stride gs elements) into shared memory (row stride ss).
// Rows >= rv or columns >= cv read as zero.  Needs 16-byte aligned row starts and cols, cv, ss
// multiples of the elements per 16 bytes (2 for complex64, 1 for complex128).
template <typename C>
__device__ __forceinline__ void tile_load(C* s, int ss, const C* g, int64_t gs, int rows, int rv, int cols, int cv) {
  constexpr int E = 16 / sizeof(C);
  const int cpr = cols / E, cvr = cv / E;
  for (int q = threadIdx.x; q < rows * cpr; q += blockDim.x) {
    const int r = q / cpr, ch = q - r * cpr;
    C* dst = s + r * ss + ch * E;
    if (r < rv && ch < cvr) {
      cp_async16(dst, g + r * gs + ch * E);
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) dst[e] = czero<C>();
    }
  }
}

// rows x cv tile from shared memory (row stride ss) to global (row stride gs), 16-byte stores
template <typename C>
__device__ __forceinline__ void tile_store(C* g, int64_t gs, const C* s, int ss, int rows, int cv) {
  constexpr int E = 16 / sizeof(C);
  const int cvr = cv / E;
  for (int q = threadIdx.x; q < rows * cvr; q += blockDim.x) {
    const int r = q / cvr, ch = q - r * cvr;
    *reinterpret_cast<int4*>(g + r * gs + ch * E) = *reinterpret_cast<const int4*>(s + r * ss + ch * E);
  }
}
// columns per z-pass tile: even (16-byte chunks), blockDim = Z * tx <= 1024 (Z <= 512)
static int z_lines_per_cta(int Z, int X) {
  int tx = 16;
  while (tx > 2 && Z * tx > 512) tx /= 2;
  return std::max(2, std::min(tx, X));
}

// ------------------------------------------------------------------------------------------
// The x and y passes run with kPassThreads threads.  Their transforms take the fully static stages
// for the usual power-of-two lengths with the line counts x_lines_per_cta / y_lines_per_cta give
// them, else the runtime stages.
constexpr int kPassThreads = 256;

// The x passes' line-major buffers: on the static path they hold element a at a + (a >> XPAD)
// with one padding element per 128 bytes (every 16 complex64, every 8 of 16-byte elements), which
// makes the first stage's stride-8 stores conflict-free.
template <typename C> __host__ __device__ constexpr int xpad_log() { return sizeof(C) == 8 ? 4 : 3; }
__host__ __device__ __forceinline__ bool x_static(int n, int nl) {
  return (n == 256 && nl == 8) || (n == 512 && nl == 4) || (n == 1024 && nl == 2);
}
// elements of a buffer holding m padded logical elements, rounded up to whole 16 bytes so that the
// second buffer (and the 16-byte tile copies of the unpadded path) stay 16-byte aligned
template <typename C> __host__ __device__ constexpr int xpad_len(int m) {
  return (m + (m >> xpad_log<C>()) + (int)(16 / sizeof(C)) - 1) / (int)(16 / sizeof(C)) * (int)(16 / sizeof(C));
}

template <int DIR, typename C>
__device__ __forceinline__ C* fft_x_lines(C* b0, C* b1, const C* tw, const FftDesc& fd, int nl) {
  constexpr int PL = xpad_log<C>();
  if (blockDim.x == kPassThreads) {
    if (fd.n == 256 && nl == 8) return fft_stages_fixed<256, 1, 8, true, DIR, kPassThreads, PL>(b0, b1, tw);
    if (fd.n == 512 && nl == 4) return fft_stages_fixed<512, 1, 4, true, DIR, kPassThreads, PL>(b0, b1, tw);
    if (fd.n == 1024 && nl == 2) return fft_stages_fixed<1024, 1, 2, true, DIR, kPassThreads, PL>(b0, b1, tw);
  }
  if constexpr (std::is_same<C, dcomplex>::value) {
    return b0;   // not reached: the double-float product is admitted only for the shapes above
  } else {
    return fft_lines<DIR>(b0, b1, tw, fd, 1, fd.n, nl, true);
  }
}

template <int DIR, typename C>
__device__ __forceinline__ C* fft_y_lines(C* b0, C* b1, const C* tw, const FftDesc& fd, int tx) {
  if (blockDim.x == kPassThreads) {
    if (fd.n == 256 && tx == 8) return fft_stages_fixed<256, 1, 8, false, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 256 && tx == 4) return fft_stages_fixed<256, 1, 4, false, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 512 && tx == 8) return fft_stages_fixed<512, 1, 8, false, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 512 && tx == 4) return fft_stages_fixed<512, 1, 4, false, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 1024 && tx == 4) return fft_stages_fixed<1024, 1, 4, false, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 1024 && tx == 2) return fft_stages_fixed<1024, 1, 2, false, DIR, kPassThreads>(b0, b1, tw);
  }
  if constexpr (std::is_same<C, dcomplex>::value) {
    return b0;   // not reached: the double-float product is admitted only for the shapes above
  } else {
    return fft_lines<DIR>(b0, b1, tw, fd, tx, 1, tx, false);
  }
}

// pass 1: fwd-x.  CTA handles `nl` consecutive lines (y fastest, then z, c, b), line-major smem.
// Each line's voxel-map row and vector offset are decoded once per CTA (XLine, after b1).
struct XLine {
  int64_t vbase;   // vmap offset of the line's (y, z) row; -1 past the last line
  int64_t xoff;    // b * ld + c * nv
  int32_t b, c;
};

__device__ __forceinline__ void decode_lines(XLine* li, int64_t l0, int nl, int64_t nlines_total, int L, int M,
                                             int y0, int ny, int z0, int nz, int64_t ld, int64_t nv) {
  for (int line = threadIdx.x; line < nl; line += blockDim.x) {
    const int64_t gl = l0 + line;
    XLine q;
    q.vbase = -1;
    q.xoff = 0;
    q.b = q.c = 0;
    if (gl < nlines_total) {
      const int64_t y = y0 + gl % ny;
      const int64_t z = z0 + (gl / ny) % nz;
      const int64_t c = (gl / ((int64_t)ny * nz)) % 5;
      const int64_t b = gl / ((int64_t)ny * nz * 5);
      q.vbase = (int64_t)L * (y + (int64_t)M * z);
      q.xoff = b * ld + c * nv;
      q.b = (int32_t)b;
      q.c = (int32_t)c;
    }
    li[line] = q;
  }
}

// t / n for the element loops (a shift when n is a power of two)
__device__ __forceinline__ int div_line(int t, int n, bool p2, int ln) { return p2 ? t >> ln : t / n; }

template <typename T>
__global__ void k_fwd_x(const double2* __restrict__ xin, int64_t ldx, const int32_t* __restrict__ vmap, int L, int M,
                        int y0, int ny, int z0, int nz, int64_t nv, int64_t nlines_total, cplx<T>* __restrict__ A,
                        FftDesc fd, const cplx<T>* __restrict__ twg, int nl) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int X = fd.n;
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* b0 = tw + X;
  C* b1 = b0 + xpad_len<C>(X * nl);
  XLine* li = reinterpret_cast<XLine*>(b1 + xpad_len<C>(X * nl));
  const bool pad = x_static(X, nl) && blockDim.x == kPassThreads;   // the layout fft_x_lines uses
  auto P = [&](int a) { return pad ? a + (a >> xpad_log<C>()) : a; };
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = twg[i];
  const int64_t l0 = (int64_t)blockIdx.x * nl;
  decode_lines(li, l0, nl, nlines_total, L, M, y0, ny, z0, nz, ldx, nv);
  __syncthreads();
  // the zero half of each line (i >= L), then the gather of i < L: every thread runs the same
  // number of gather rounds, so that a warp none of whose elements is a voxel skips the loads and
  // the complex128 -> complex64 conversions (FP64-pipe work on GB300) as a whole
  const int XL = X - L;
  for (int t = threadIdx.x; t < XL * nl; t += blockDim.x) {
    const int line = t / XL;
    b0[P(line * X + L + (t - line * XL))] = czero<C>();
  }
  const bool p2 = (L & (L - 1)) == 0;
  const int ll = __ffs(L) - 1;
  const int tot = L * nl;
  for (int base = 0; base < tot; base += 4 * blockDim.x) {
    int32_t vid[4];
    int64_t off[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {     // independent voxel-map loads
      const int t = base + threadIdx.x + u * blockDim.x;
      vid[u] = -1;
      off[u] = 0;
      if (t < tot) {
        const int line = div_line(t, L, p2, ll), i = t - line * L;
        const XLine q = li[line];
        if (q.vbase >= 0) {
          vid[u] = vmap[i + q.vbase];
          off[u] = q.xoff;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int t = base + threadIdx.x + u * blockDim.x;
      C v = czero<C>();
      if (__any_sync(0xffffffffu, vid[u] >= 0)) {
        if (vid[u] >= 0) v = to_c(xin[off[u] + vid[u]], C());
      }
      if (t < tot) {
        const int line = div_line(t, L, p2, ll);
        b0[P(line * X + (t - line * L))] = v;
      }
    }
  }
  __syncthreads();
  C* r = fft_x_lines<-1>(b0, b1, tw, fd, nl);
  const int rows = (nlines_total - l0 < nl) ? (int)(nlines_total - l0) : nl;
  if (pad) {   // element by element out of the padded buffer (coalesced on the global side)
    C* Ag = A + l0 * X;
    for (int q = threadIdx.x; q < rows * X; q += blockDim.x) Ag[q] = r[P(q)];
  } else {
    tile_store(A + l0 * X, X, r, X, rows, X);
  }
}

// pass 2 / 4: FFT along y.  Rows of `nin` input (index < nin), `nout` output rows written.
// src: [plane][nin_rows_stride][X], dst: [plane][nout_stride][X]; CTA: `tx` consecutive kx of one plane.
// The nin source rows enter the transform at rows in_off..; result rows out_off.. are stored.
template <typename T, int DIR>
__global__ void k_pass_y(const cplx<T>* __restrict__ src, int src_rows, int nin, cplx<T>* __restrict__ dst,
                         int dst_rows, int nout, int X, FftDesc fd, const cplx<T>* __restrict__ twg, int tx,
                         int in_off, int out_off) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Y = fd.n;
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* b0 = tw + Y;
  C* b1 = b0 + Y * tx;
  for (int i = threadIdx.x; i < Y; i += blockDim.x) tw[i] = twg[i];
  const int kx0 = blockIdx.x * tx;
  const int64_t plane = blockIdx.y;
  const C* s = src + plane * src_rows * (int64_t)X;
  C* d = dst + plane * dst_rows * (int64_t)X;
  const int cv = min(tx, X - kx0);
  for (int q = threadIdx.x; q < in_off * tx; q += blockDim.x) b0[q] = czero<C>();
  tile_load(b0 + in_off * tx, tx, s + kx0, X, Y - in_off, nin, tx, cv);
  cp_async_wait_all();
  __syncthreads();
  C* r = fft_y_lines<DIR>(b0, b1, tw, fd, tx);
  tile_store(d + kx0, X, r + out_off * tx, tx, nout, cv);
}

// pass 2 / 4 for Y = 256, 512, 1024 in registers: Y = R1 R2 (R2 = 32 for 512 and 1024, 16 for 256),
// a CTA takes NC consecutive kx columns of one plane (NC = 128 bytes of row: 16 complex64 values, 8
// complex128 or double-float values).  Row n = j + R2 m, output k = k1 + R1 k2:
//   step 1: thread (c, j) gathers x[j + R2 m], m < R1 (rows outside the input window are zero and not
//           read), transforms over m (R1 points: A_j[k1]), multiplies by w_Y^(j k1) and stores the
//           products in shared memory;
//   step 2: thread (c, k1) transforms them over j (R2 points): X[k1 + R1 k2]; rows outside the output
//           window are not stored.
// One shared-memory exchange per transform (the ping-pong stages of k_pass_y take log8 Y of them).
template <typename C, int DIR, int R1, int R2, int NC>
__global__ void __launch_bounds__(NC * R2)
    k_pass_y_reg(const C* __restrict__ src, int src_rows, int nin, C* __restrict__ dst, int dst_rows, int nout, int X,
                 const C* __restrict__ twg, int in_off, int out_off) {
  constexpr int Y = R1 * R2, NT = NC * R2;
  static_assert(R1 <= R2, "step 2 runs R1 of the R2 thread rows");
  extern __shared__ __align__(16) unsigned char yr_raw[];
  C* tw = reinterpret_cast<C*>(yr_raw);   // tw[i] = exp(-2 pi i i / Y)
  C* T = tw + Y;                            // T[(k1 * R2 + j) * NC + c]
  for (int i = threadIdx.x; i < Y; i += NT) tw[i] = twg[i];
  const int c = threadIdx.x % NC;
  const int kx0 = blockIdx.x * NC;
  const bool col_ok = kx0 + c < X;
  const int64_t plane = blockIdx.y;
  const C* s = src + plane * src_rows * (int64_t)X + kx0 + c;
  C* d = dst + plane * dst_rows * (int64_t)X + kx0 + c;
  __syncthreads();
  {
    const int j = threadIdx.x / NC;
    C v[R1];
#pragma unroll
    for (int m = 0; m < R1; ++m) {
      const int r = j + R2 * m - in_off;
      v[m] = (col_ok && r >= 0 && r < nin) ? s[(int64_t)r * X] : czero<C>();
    }
    dif_pruned<Y, R1, R1, DIR>(v, tw);   // v[p] = A_j[bitrev(p)]
#pragma unroll
    for (int p = 0; p < R1; ++p) {
      const int k1 = bit_reverse<ilog2c(R1)>(p);
      const C w = tw[j * k1];
      T[(k1 * R2 + j) * NC + c] = DIR < 0 ? cmul(v[p], w) : cmulc(v[p], w);
    }
  }
  __syncthreads();
  for (int k1 = threadIdx.x / NC; k1 < R1; k1 += NT / NC) {
    C v[R2];
#pragma unroll
    for (int j = 0; j < R2; ++j) v[j] = T[(k1 * R2 + j) * NC + c];
    dif_pruned<Y, R2, R2, DIR>(v, tw);   // v[p] = X[k1 + R1 bitrev(p)]
#pragma unroll
    for (int p = 0; p < R2; ++p) {
      const int k = k1 + R1 * bit_reverse<ilog2c(R2)>(p) - out_off;
      if (col_ok && k >= 0 && k < nout) d[(int64_t)k * X] = v[p];
    }
  }
}

template <typename C, int DIR, int R1, int R2, int SEG = 128>
static void launch_pass_y_reg(const C* src, int src_rows, int nin, C* dst, int dst_rows, int nout, int X,
                              unsigned planes, const C* tw, int in_off, int out_off, cudaStream_t st) {
  constexpr int NC = SEG / (int)sizeof(C);   // columns per block: SEG bytes of each row
  constexpr size_t sm = (size_t)R1 * R2 * (NC + 1) * sizeof(C);
  static_assert(sm <= 227 * 1024, "y-pass shared memory");
  allow_dyn_smem(k_pass_y_reg<C, DIR, R1, R2, NC>, sm);
  dim3 grid((unsigned)ceil_div(X, NC), planes);
  k_pass_y_reg<C, DIR, R1, R2, NC><<<grid, NC * R2, sm, st>>>(src, src_rows, nin, dst, dst_rows, nout, X, tw, in_off,
                                                              out_off);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

// the register y-pass when Y is 256, 512 or 1024; false otherwise.  narrow: 64-byte row segments
// (half the columns per block: half the shared memory and threads, so more blocks fit an SM)
template <int DIR, typename C>
static bool pass_y_reg(int Y, const C* src, int src_rows, int nin, C* dst, int dst_rows, int nout, int X,
                       unsigned planes, const C* tw, int in_off, int out_off, cudaStream_t st, bool narrow = false) {
  if (narrow) {
    switch (Y) {
      case 256: launch_pass_y_reg<C, DIR, 16, 16, 64>(src, src_rows, nin, dst, dst_rows, nout, X, planes, tw, in_off, out_off, st); return true;
      case 512: launch_pass_y_reg<C, DIR, 16, 32, 64>(src, src_rows, nin, dst, dst_rows, nout, X, planes, tw, in_off, out_off, st); return true;
      case 1024: launch_pass_y_reg<C, DIR, 32, 32, 64>(src, src_rows, nin, dst, dst_rows, nout, X, planes, tw, in_off, out_off, st); return true;
      default: return false;
    }
  }
  switch (Y) {
    case 256: launch_pass_y_reg<C, DIR, 16, 16>(src, src_rows, nin, dst, dst_rows, nout, X, planes, tw, in_off, out_off, st); return true;
    case 512: launch_pass_y_reg<C, DIR, 16, 32>(src, src_rows, nin, dst, dst_rows, nout, X, planes, tw, in_off, out_off, st); return true;
    case 1024: launch_pass_y_reg<C, DIR, 32, 32>(src, src_rows, nin, dst, dst_rows, nout, X, planes, tw, in_off, out_off, st); return true;
    default: return false;
  }
}

// The 13 distinct products of the 5 current spectra with the 7 tensor components at one point
// (lse_matvect_mult.m:57-86), in place: (Jx, Jy, Jz, J2D, J3D) -> their operator images.
template <typename C>
__device__ __forceinline__ void tensor_apply(const C* g, C& jx, C& jy, C& jz, C& j2, C& j3) {
  const C a = cmul(g[1], jx);             // G2 Jx
  const C bb = cmul(g[2], jy);            // G3 Jy
  const C o1 = cadd(cmul(g[0], jx), cmul(g[1], cadd(j2, j3)));
  const C o2 = cadd(cmul(g[0], jy), cmul(g[2], csub(j2, j3)));
  const C o3 = cadd(cmul(g[0], jz), cmul(g[4], j3));
  const C o4 = cadd(csub(cneg(a), bb), cadd(cmul(g[3], j2), cmul(g[5], j3)));
  const C o5 = cadd(cadd(csub(bb, a), cneg(cmul(g[4], jz))), cadd(cmul(g[5], j2), cmul(g[6], j3)));
  jx = o1;
  jy = o2;
  jz = o3;
  j2 = o4;
  j3 = o5;
}

// tensor_apply for a spectrum whose components 0, 3, 5, 6 are real and 1, 2, 4 imaginary: g[k] is
// the real part or the imaginary part, and each product is two real multiplications
template <typename C, typename T>
__device__ __forceinline__ void tensor_apply_ri(const T* g, C& jx, C& jy, C& jz, C& j2, C& j3) {
  auto rm = [](T s, const C& v) { C r; r.x = s * v.x; r.y = s * v.y; return r; };    // s v
  auto im = [](T s, const C& v) { C r; r.x = -s * v.y; r.y = s * v.x; return r; };   // i s v
  const C a = im(g[1], jx);               // G2 Jx
  const C bb = im(g[2], jy);              // G3 Jy
  const C o1 = cadd(rm(g[0], jx), im(g[1], cadd(j2, j3)));
  const C o2 = cadd(rm(g[0], jy), im(g[2], csub(j2, j3)));
  const C o3 = cadd(rm(g[0], jz), im(g[4], j3));
  const C o4 = cadd(csub(cneg(a), bb), cadd(rm(g[3], j2), rm(g[5], j3)));
  const C o5 = cadd(cadd(csub(bb, a), cneg(im(g[4], jz))), cadd(rm(g[5], j2), rm(g[6], j3)));
  jx = o1;
  jy = o2;
  jz = o3;
  j2 = o4;
  j3 = o5;
}

// pass 3: z-FFT, tensor product, inverse z-FFT.  B[b][c][z<N][ky][kx] in place.
// blockDim = Z * tx; thread (kz, tx) keeps the 7 tensor values of its point in registers.
template <typename T>
__global__ void k_zpass(cplx<T>* __restrict__ Bf, const cplx<T>* __restrict__ tens, int z0, int nz, int Y, int X,
                        int nrhs, FftDesc fd, const cplx<T>* __restrict__ twg, int tx) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int Z = fd.n;
  const int nl = 5 * tx;  // lines: c * tx + t
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* b0 = tw + Z;
  C* b1 = b0 + Z * nl;
  for (int i = threadIdx.x; i < Z; i += blockDim.x) tw[i] = twg[i];
  const int kx0 = blockIdx.x * tx;
  const int ky = blockIdx.y;
  const int my_t = threadIdx.x % tx;
  const int my_kz = threadIdx.x / tx;
  const int my_kx = kx0 + my_t;
  C g[7];
  if (my_kz < Z && my_kx < X) {
#pragma unroll
    for (int k = 0; k < 7; ++k) g[k] = tens[(((int64_t)ky * Z + my_kz) * 7 + k) * X + my_kx];
  } else {
#pragma unroll
    for (int k = 0; k < 7; ++k) g[k] = czero<C>();
  }
  const int64_t plane = (int64_t)Y * X;       // one z row of one component
  const int64_t comp = (int64_t)nz * plane;   // one component of one RHS
  for (int b = 0; b < nrhs; ++b) {
    C* base = Bf + (int64_t)b * 5 * comp + (int64_t)ky * X;
    const int cv = min(tx, X - kx0);
    for (int q = threadIdx.x; q < z0 * nl; q += blockDim.x) b0[q] = czero<C>();   // rows below the voxels
#pragma unroll
    for (int c = 0; c < 5; ++c)
      tile_load(b0 + c * tx + z0 * nl, nl, base + c * comp + kx0, plane, Z - z0, nz, tx, cv);
    cp_async_wait_all();
    __syncthreads();
    C* f = fft_lines<-1>(b0, b1, tw, fd, nl, 1, nl, false);
    if (my_kz < Z) {
      C* p = f + my_kz * nl + my_t;
      tensor_apply(g, p[0], p[tx], p[2 * tx], p[3 * tx], p[4 * tx]);
    }
    __syncthreads();
    C* other = (f == b0) ? b1 : b0;
    C* r = fft_lines<+1>(f, other, tw, fd, nl, 1, nl, false);
#pragma unroll
    for (int c = 0; c < 5; ++c) tile_store(base + c * comp + kx0, plane, r + c * tx + z0 * nl, nl, nz, cv);
    __syncthreads();
  }
}

// pass 3 for Z = 8, 16, 32, 64: the z transform of each column in registers, two threads per
// column.  The nz voxel rows enter the transform at rows 0.. (circular convolution is shift
// invariant), so the forward transform reads only NZ >= nz leading rows and the inverse forms only
// the first NZ rows (pruned at compile time).  NZ <= Z / 2, so the first decimation-in-frequency
// stage only copies (lower half) or twiddles (upper half) the inputs: lane half h = 0 takes the
// lower half, h = 1 the upper, and each runs the remaining Z/2-point transform alone.  The last
// decimation-in-time stage of the inverse needs both halves at each output row: the two lanes of a
// column (lane and lane ^ 16) trade half of their rows by shuffle and each forms half of the outputs.
// The operations and their order are those of the full-column transform (dif_pruned / dit_pruned
// of length Z), so the results are the same.
// Block: 5 warps (warp = component) over 16 columns of one ky row (lane = column + 16 h); the five
// spectra of a point meet in shared memory for the tensor product, and the block's tensor values
// (the same for every RHS of the batch) are staged in shared memory once.
constexpr int kZregCols = 16;

// storage <-> arithmetic type of the z-pass (identity, or complex128 storage with double-float
// arithmetic)
__device__ __forceinline__ float2 zload(float2 v, float2) { return v; }
__device__ __forceinline__ double2 zload(double2 v, double2) { return v; }
__device__ __forceinline__ dcomplex zload(double2 v, dcomplex) { return to_c(v, dcomplex()); }
__device__ __forceinline__ float2 zstore(float2 v, float2) { return v; }
__device__ __forceinline__ double2 zstore(double2 v, double2) { return v; }
__device__ __forceinline__ double2 zstore(dcomplex v, double2) { return to_d(v); }
__device__ __forceinline__ dcomplex zload(dcomplex v, dcomplex) { return v; }
__device__ __forceinline__ dcomplex zstore(dcomplex v, dcomplex) { return v; }

// a complex value from lane ^ m
__device__ __forceinline__ float2 shfl_xor_c(float2 v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}
__device__ __forceinline__ double2 shfl_xor_c(double2 v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}
__device__ __forceinline__ dcomplex shfl_xor_c(dcomplex v, int m) {
  v.x.hi = __shfl_xor_sync(0xffffffffu, v.x.hi, m);
  v.x.lo = __shfl_xor_sync(0xffffffffu, v.x.lo, m);
  v.y.hi = __shfl_xor_sync(0xffffffffu, v.y.hi, m);
  v.y.lo = __shfl_xor_sync(0xffffffffu, v.y.lo, m);
  return v;
}

template <typename T, int Z, typename GT>
__host__ __device__ constexpr size_t zpass_reg_smem() {
  return (size_t)(Z + 5 * Z * kZregCols) * sizeof(cplx<T>) + (size_t)Z * 7 * kZregCols * sizeof(GT);
}

template <typename T, int Z, int NZ, typename ST = cplx<T>, typename GT = cplx<T>>
__global__ void __launch_bounds__(5 * 32)
    k_zpass_reg(ST* __restrict__ Bf, const GT* __restrict__ tens, int nz, int Y, int X, int nrhs,
                const cplx<T>* __restrict__ twg) {
  using C = cplx<T>;
  constexpr int H = Z / 2;
  constexpr int HN = NZ / 2;                 // output rows formed by each lane of a column
  constexpr int BITS = ilog2c(Z);
  constexpr int NC = kZregCols;
  static_assert(Z == 8 || Z == 16 || Z == 32 || Z == 64, "register z-pass lengths");
  static_assert(NZ >= 2 && NZ <= H, "pruned rows");
  constexpr bool kRI = sizeof(GT) < sizeof(C);   // real/imaginary tensor: one T per component
  extern __shared__ __align__(16) unsigned char zr_raw[];
  C* tw = reinterpret_cast<C*>(zr_raw);
  C* S = tw + Z;                                             // S[(c * Z + p) * NC + col]
  GT* G = reinterpret_cast<GT*>(S + 5 * Z * NC);             // G[(p * 7 + k) * NC + col]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = lane & (NC - 1);
  const bool hi = lane >= NC;
  for (int i = threadIdx.x; i < Z; i += blockDim.x) tw[i] = twg[i];
  const int ky = blockIdx.y;
  const int kx0 = blockIdx.x * NC;
  // the tensor values of the block's points, position p holding kz = bitrev(p)
  for (int i = threadIdx.x; i < Z * 7 * NC; i += blockDim.x) {
    const int c = i % NC, k = (i / NC) % 7, p = i / (7 * NC);
    const int kz = bit_reverse<BITS>(p);
    G[i] = (kx0 + c < X) ? tens[(((int64_t)ky * Z + kz) * 7 + k) * X + kx0 + c] : GT{};
  }
  const int kx = kx0 + col;
  const bool col_ok = kx < X;
  const int64_t plane = (int64_t)Y * X;       // one z row of one component
  const int64_t comp = (int64_t)nz * plane;   // one component of one RHS
  __syncthreads();
  for (int b = 0; b < nrhs; ++b) {
    ST* base = Bf + ((int64_t)b * 5 + warp) * comp + (int64_t)ky * X + kx;
    {
      C v[H];
#pragma unroll
      for (int n = 0; n < H; ++n) v[n] = czero<C>();
#pragma unroll
      for (int n = 0; n < NZ; ++n)
        if (n < nz && col_ok) v[n] = zload(base[n * plane], C());
      // first decimation-in-frequency stage (upper input half zero): the upper output half is the
      // twiddled input
#pragma unroll
      for (int n = 0; n < NZ; ++n)
        if (hi) v[n] = tw_mul<Z, Z, -1>(v[n], n, tw);
      dif_pruned<Z, H, NZ, -1>(v, tw);
#pragma unroll
      for (int q = 0; q < H; ++q) S[(warp * Z + (hi ? H : 0) + q) * NC + col] = v[q];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < Z * NC; i += blockDim.x) {
      const int p = i / NC, c = i % NC;
      GT g[7];
#pragma unroll
      for (int k = 0; k < 7; ++k) g[k] = G[(p * 7 + k) * NC + c];
      C* q = S + p * NC + c;
      constexpr int cs = Z * NC;
      if constexpr (kRI)
        tensor_apply_ri(g, q[0], q[cs], q[2 * cs], q[3 * cs], q[4 * cs]);
      else
        tensor_apply(g, q[0], q[cs], q[2 * cs], q[3 * cs], q[4 * cs]);
    }
    __syncthreads();
    {
      C v[H];
#pragma unroll
      for (int q = 0; q < H; ++q) v[q] = S[(warp * Z + (hi ? H : 0) + q) * NC + col];
      dit_pruned<Z, H, NZ, +1>(v, tw);
      // last decimation-in-time stage, rows k < NZ: out[k] = X0[k] + w^k X1[k] (X0: lower half,
      // X1: upper); the lower lane forms rows 0..HN-1, the upper lane rows HN..NZ-1
#pragma unroll
      for (int i = 0; i < HN; ++i) {
        const C mine = hi ? v[HN + i] : v[i];
        const C other = shfl_xor_c(hi ? v[i] : v[HN + i], NC);   // X0[HN + i] to the upper, X1[i] to the lower
        const C o = hi ? cadd(other, tw_mul<Z, Z, +1>(mine, HN + i, tw)) : cadd(mine, tw_mul<Z, Z, +1>(other, i, tw));
        const int k = (hi ? HN : 0) + i;
        if (k < nz && col_ok) base[k * plane] = zstore(o, ST());
      }
    }
    __syncthreads();   // S is rewritten by the next RHS
  }
}

template <typename T, int Z, int NZ, typename ST, typename GT>
static void launch_zpass_reg(ST* Bf, const GT* tens, int nz, int Y, int X, int B, const cplx<T>* tw,
                             cudaStream_t st) {
  constexpr size_t sm = zpass_reg_smem<T, Z, GT>();
  static_assert(sm <= 227 * 1024, "z-pass shared memory");
  allow_dyn_smem(k_zpass_reg<T, Z, NZ, ST, GT>, sm);
  dim3 grid((unsigned)ceil_div(X, kZregCols), (unsigned)Y);
  k_zpass_reg<T, Z, NZ, ST, GT><<<grid, 5 * 32, sm, st>>>(Bf, tens, nz, Y, X, B, tw);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

// pass 3 alternative for Z = 8, 16, 32 (the autotuner's z_variant 2): one thread transforms a whole
// column of one component in registers (the same pruned transforms), 5 warps over 32 columns of one
// ky row, the thread's tensor values held in registers for all RHS when they fit.  It keeps more
// columns per block and fewer exchanges than the two-lane pass, and pays for it in registers as Z
// grows (255 at Z = 32).
constexpr int kZcolCols = 32;

template <typename T, int Z, int NZ, typename ST = cplx<T>, typename GT = cplx<T>>
__global__ void __launch_bounds__(5 * kZcolCols)
    k_zpass_col(ST* __restrict__ Bf, const GT* __restrict__ tens, int nz, int Y, int X, int nrhs,
                const cplx<T>* __restrict__ twg) {
  using C = cplx<T>;
  constexpr int BITS = Z == 8 ? 3 : (Z == 16 ? 4 : 5);
  static_assert(Z == 8 || Z == 16 || Z == 32, "register z-pass lengths");
  extern __shared__ __align__(16) unsigned char zr_raw[];
  C* tw = reinterpret_cast<C*>(zr_raw);
  C* S = tw + Z;   // S[(c * Z + p) * 32 + lane]: component c, transform position p
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < Z; i += blockDim.x) tw[i] = twg[i];
  const int ky = blockIdx.y;
  const int kx = blockIdx.x * kZcolCols + lane;
  const bool col_ok = kx < X;
  const int64_t plane = (int64_t)Y * X;       // one z row of one component
  const int64_t comp = (int64_t)nz * plane;   // one component of one RHS
  // the tensor values of this thread's positions p = warp + 5 q, loaded once for all RHS when
  // they fit in registers (they are the same for every RHS of the batch)
  constexpr int Q = (Z + 4) / 5;
  constexpr bool kRI = sizeof(GT) < sizeof(C);   // real/imaginary tensor: one T per component
  constexpr bool kHoist = sizeof(GT) * 7 * Q <= 256;
  GT gq[kHoist ? Q : 1][7];
  if constexpr (kHoist) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int p = warp + 5 * q;
      const int kz = bit_reverse<BITS>(p < Z ? p : 0);
#pragma unroll
      for (int k = 0; k < 7; ++k)
        gq[q][k] = (col_ok && p < Z) ? tens[(((int64_t)ky * Z + kz) * 7 + k) * X + kx] : GT{};
    }
  }
  __syncthreads();
  for (int b = 0; b < nrhs; ++b) {
    ST* base = Bf + (int64_t)b * 5 * comp + (int64_t)ky * X + kx;
    {
      C v[Z];
#pragma unroll
      for (int i = 0; i < Z; ++i) v[i] = czero<C>();
#pragma unroll
      for (int i = 0; i < NZ; ++i)
        if (i < nz && col_ok) v[i] = zload(base[warp * comp + i * plane], C());
      dif_pruned<Z, Z, NZ, -1>(v, tw);
#pragma unroll
      for (int p = 0; p < Z; ++p) S[(warp * Z + p) * kZcolCols + lane] = v[p];
    }
    __syncthreads();
    if constexpr (kHoist) {
#pragma unroll
      for (int qi = 0; qi < Q; ++qi) {
        const int p = warp + 5 * qi;
        if (p < Z) {
          C* q = S + p * kZcolCols + lane;
          constexpr int cs = Z * kZcolCols;
          if constexpr (kRI)
            tensor_apply_ri(gq[qi], q[0], q[cs], q[2 * cs], q[3 * cs], q[4 * cs]);
          else
            tensor_apply(gq[qi], q[0], q[cs], q[2 * cs], q[3 * cs], q[4 * cs]);
        }
      }
    } else {
      for (int p = warp; p < Z; p += 5) {   // position p holds kz = bitrev(p)
        const int kz = bit_reverse<BITS>(p);
        GT g[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) g[k] = col_ok ? tens[(((int64_t)ky * Z + kz) * 7 + k) * X + kx] : GT{};
        C* q = S + p * kZcolCols + lane;
        constexpr int cs = Z * kZcolCols;
        if constexpr (kRI)
          tensor_apply_ri(g, q[0], q[cs], q[2 * cs], q[3 * cs], q[4 * cs]);
        else
          tensor_apply(g, q[0], q[cs], q[2 * cs], q[3 * cs], q[4 * cs]);
      }
    }
    __syncthreads();
    {
      C v[Z];
#pragma unroll
      for (int p = 0; p < Z; ++p) v[p] = S[(warp * Z + p) * kZcolCols + lane];
      dit_pruned<Z, Z, NZ, +1>(v, tw);
#pragma unroll
      for (int i = 0; i < NZ; ++i)
        if (i < nz && col_ok) base[warp * comp + i * plane] = zstore(v[i], ST());
    }
    __syncthreads();   // S is rewritten by the next RHS
  }
}

template <typename T, int Z, int NZ, typename ST, typename GT>
static void launch_zpass_col(ST* Bf, const GT* tens, int nz, int Y, int X, int B, const cplx<T>* tw,
                             cudaStream_t st) {
  const size_t sm = (size_t)(Z + 5 * Z * kZcolCols) * sizeof(cplx<T>);
  allow_dyn_smem(k_zpass_col<T, Z, NZ, ST, GT>, sm);
  dim3 grid((unsigned)ceil_div(X, kZcolCols), (unsigned)Y);
  k_zpass_col<T, Z, NZ, ST, GT><<<grid, 5 * kZcolCols, sm, st>>>(Bf, tens, nz, Y, X, B, tw);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

// true when the register z-pass handles this length (Z = 8, 16, 32, and 64 outside the
// double-float product; nz <= Z / 2 always holds); T is the arithmetic type, ST the storage type of
// the spectra
template <typename T, typename ST = cplx<T>, typename GT = cplx<T>>
static bool zpass_reg(int Z, int nz, ST* Bf, const GT* tens, int Y, int X, int B, const cplx<T>* tw,
                      cudaStream_t st) {
  int nzb = 2;
  while (nzb < nz) nzb *= 2;
  switch (Z * 100 + nzb) {
    case 802: launch_zpass_reg<T, 8, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 804: launch_zpass_reg<T, 8, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 1602: launch_zpass_reg<T, 16, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 1604: launch_zpass_reg<T, 16, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 1608: launch_zpass_reg<T, 16, 8>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3202: launch_zpass_reg<T, 32, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3204: launch_zpass_reg<T, 32, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3208: launch_zpass_reg<T, 32, 8>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3216: launch_zpass_reg<T, 32, 16>(Bf, tens, nz, Y, X, B, tw, st); return true;
    default: break;
  }
  if constexpr (!std::is_same<T, dfloat>::value) {
    switch (Z * 100 + nzb) {
      case 6402: launch_zpass_reg<T, 64, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
      case 6404: launch_zpass_reg<T, 64, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
      case 6408: launch_zpass_reg<T, 64, 8>(Bf, tens, nz, Y, X, B, tw, st); return true;
      case 6416: launch_zpass_reg<T, 64, 16>(Bf, tens, nz, Y, X, B, tw, st); return true;
      case 6432: launch_zpass_reg<T, 64, 32>(Bf, tens, nz, Y, X, B, tw, st); return true;
      default: break;
    }
  }
  return false;
}

// the one-thread-per-column z-pass for Z = 8, 16, 32; false otherwise
template <typename T, typename ST = cplx<T>, typename GT = cplx<T>>
static bool zpass_col(int Z, int nz, ST* Bf, const GT* tens, int Y, int X, int B, const cplx<T>* tw,
                      cudaStream_t st) {
  int nzb = 2;
  while (nzb < nz) nzb *= 2;
  switch (Z * 100 + nzb) {
    case 802: launch_zpass_col<T, 8, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 804: launch_zpass_col<T, 8, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 1602: launch_zpass_col<T, 16, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 1604: launch_zpass_col<T, 16, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 1608: launch_zpass_col<T, 16, 8>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3202: launch_zpass_col<T, 32, 2>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3204: launch_zpass_col<T, 32, 4>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3208: launch_zpass_col<T, 32, 8>(Bf, tens, nz, Y, X, B, tw, st); return true;
    case 3216: launch_zpass_col<T, 32, 16>(Bf, tens, nz, Y, X, B, tw, st); return true;
    default: return false;
  }
}

// the z-pass of the launch choice: the one-thread-per-column pass when z_variant is 2 and it takes the
// length, else the two-lane register pass
template <typename T, typename ST = cplx<T>, typename GT = cplx<T>>
static bool zpass_any(int z_variant, int Z, int nz, ST* Bf, const GT* tens, int Y, int X, int B, const cplx<T>* tw,
                      cudaStream_t st) {
  if (z_variant == 2 && zpass_col<T, ST, GT>(Z, nz, Bf, tens, Y, X, B, tw, st)) return true;
  return zpass_reg<T, ST, GT>(Z, nz, Bf, tens, Y, X, B, tw, st);
}

// pass 5: inverse x-FFT, crop, diagonal term, scatter.
template <typename T>
__global__ void k_inv_x(const cplx<T>* __restrict__ A, const int32_t* __restrict__ vmap, int L, int M, int y0,
                        int ny, int z0, int nz, int64_t nv, int64_t nlines_total, const double2* __restrict__ xin,
                        int64_t ldx,
                        double2* __restrict__ yout, int64_t ldy, const double2* __restrict__ scale,
                        const double2* __restrict__ zdiag, int64_t zstride, double inv_dx, FftDesc fd,
                        const cplx<T>* __restrict__ twg, int nl) {
  using C = cplx<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int X = fd.n;
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* b0 = tw + X;
  C* b1 = b0 + xpad_len<C>(X * nl);
  XLine* li = reinterpret_cast<XLine*>(b1 + xpad_len<C>(X * nl));
  const bool pad = x_static(X, nl) && blockDim.x == kPassThreads;   // the layout fft_x_lines uses
  auto P = [&](int a) { return pad ? a + (a >> xpad_log<C>()) : a; };
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = twg[i];
  const int64_t l0 = (int64_t)blockIdx.x * nl;
  const int rows_valid = (nlines_total - l0 < nl) ? (int)(nlines_total - l0) : nl;
  float2* sline = reinterpret_cast<float2*>(li + nl);   // the line's RHS scale in FP32 (complex64 product)
  decode_lines(li, l0, nl, nlines_total, L, M, y0, ny, z0, nz, ldx, nv);
  if constexpr (sizeof(T) == 4) {
    for (int line = threadIdx.x; line < nl; line += blockDim.x) sline[line] = to_c(scale[li[line].b], float2());
  }
  if (pad) {   // element by element into the padded buffer (rows past the last line read as zero)
    const C* Ag = A + l0 * X;
    for (int q = threadIdx.x; q < nl * X; q += blockDim.x) b0[P(q)] = q < rows_valid * X ? Ag[q] : czero<C>();
  } else {
    tile_load(b0, X, A + l0 * X, X, nl, rows_valid, X, X);
    cp_async_wait_all();
  }
  __syncthreads();
  C* r = fft_x_lines<+1>(b0, b1, tw, fd, nl);
  const bool p2 = (L & (L - 1)) == 0;
  const int ll = __ffs(L) - 1;
  for (int t = threadIdx.x; t < L * nl; t += blockDim.x) {
    const int line = div_line(t, L, p2, ll), i = t - line * L;
    const XLine q = li[line];
    if (q.vbase < 0) continue;
    const int64_t b = q.b, c = q.c;
    const int32_t vid = vmap[i + q.vbase];
    if (vid < 0) continue;
    const double2 zz = zdiag[b * zstride + vid];
    const double2 xj = xin[b * ldx + c * nv + vid];
    const double ck = (c < 3 ? 1.0 : (c == 3 ? 1.0 / 6.0 : 0.5)) * inv_dx;
    if constexpr (sizeof(T) == 4) {
      // complex64 product: the diagonal term in FP32 too (rounding ~1e-7, below the complex64
      // transform's own error), which keeps GB300's FP64 pipe to the conversions
      const float2 conv = r[P(line * X + i)];
      const float2 sf = sline[line], zf = to_c(zz, float2()), xf = to_c(xj, float2());
      const float2 d = cmul(zf, xf);
      const float ckf = (float)ck;
      float2 o = cmul(sf, conv);
      o.x = fmaf(ckf, d.x, o.x);
      o.y = fmaf(ckf, d.y, o.y);
      yout[b * ldy + c * nv + vid] = make_double2((double)o.x, (double)o.y);
    } else {
      const double2 conv = to_d(r[P(line * X + i)]);
      double2 out = cmul(scale[b], conv);
      out = cadd(out, cscale(cmul(zz, xj), ck));
      yout[b * ldy + c * nv + vid] = out;
    }
  }
}

// the register z-pass in double-float arithmetic on pair storage (vh_conv_df_z.cu)
bool zpass_df(int z_variant, int Z, int nz, dcomplex* Bf, const dfloat* tens_ri, int Y, int X, int B,
              const dcomplex* tw, cudaStream_t st);

// true when the double-float product handles the plan: a real/imaginary spectrum, x and y lengths and
// line counts with compile-time stages and a register z-pass length (else the complex128 product)
inline bool conv_df_supported(const ConvPlan& p) {
  if (!p.ri) return false;
  auto p2 = [](int n) { return n == 256 || n == 512 || n == 1024; };
  const int nl = x_lines_per_cta(p.X, TileCfg<dfloat>::target);
  const int tx = y_lines_per_cta(p.Y, p.X, true);
  const bool x_ok = p2(p.X) && nl == 2048 / p.X;
  const bool y_ok = (p.Y == 256 || p.Y == 512) ? tx == 4 : (p.Y == 1024 && tx == 2);
  int nzb = 2;
  while (nzb < p.nz) nzb *= 2;
  const bool z_ok = (p.Z == 8 && nzb <= 4) || (p.Z == 16 && nzb <= 8) || (p.Z == 32 && nzb <= 16);
  return x_ok && y_ok && z_ok;
}

// the tensor spectrum and twiddle tables of each arithmetic type: complex64, complex128, and the
// double-float pairs of the PREC_DF product (spectra stored as pairs between its passes)
template <typename T> struct ConvTables;
template <> struct ConvTables<float> {
  static const float2* tens(const ConvPlan& p) { return p.tens32; }
  static const float2* tw(const ConvPlan& p, int a) { return p.tw32[a]; }
};
template <> struct ConvTables<double> {
  static const double2* tens(const ConvPlan& p) { return p.tens64; }
  static const double2* tw(const ConvPlan& p, int a) { return p.tw64[a]; }
};
template <> struct ConvTables<dfloat> {
  // (the real/imaginary pairs: pass 3 reads them as dfloat; this pointer is only tested for null)
  static const dcomplex* tens(const ConvPlan& p) { return static_cast<const dcomplex*>(p.tensdf); }
  static const dcomplex* tw(const ConvPlan& p, int a) {
    return static_cast<const dcomplex*>(a == 0 ? p.twxdf : (a == 1 ? p.twydf : p.twdf));
  }
};

template <typename T>
static void conv_apply_t(ConvPlan& p, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                         const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st) {
  using C = cplx<T>;
  const bool dbl = sizeof(C) == 16;
  C* A = reinterpret_cast<C*>(p.scratchA);
  C* Bf = reinterpret_cast<C*>(p.scratchB);
  const C* tens = ConvTables<T>::tens(p);
  const C* twp[3] = {ConvTables<T>::tw(p, 0), ConvTables<T>::tw(p, 1), ConvTables<T>::tw(p, 2)};
  VH_REQUIRE(tens != nullptr && twp[0] && twp[1] && twp[2], ERR_BAD_ARG, "tensor for this precision was not built");
  const int X = p.X, Y = p.Y, Z = p.Z, L = p.L, M = p.M;
  const int y0 = p.y0, ny = p.ny, z0 = p.z0, nz = p.nz;
  VH_REQUIRE(ny > 0 && nz > 0, ERR_BAD_ARG, "FFT convolution of a geometry without voxels");
  // pass 1
  bool x_warp = false;
  if constexpr (std::is_same<T, float>::value) {
    if (p.x_variant_now == 1) x_warp = xpass_warp_fwd(p, B, x, ldx, A, st);
  }
  if (!x_warp) {
    const int nl = x_lines_per_cta(X, TileCfg<T>::target);
    const int64_t lines = (int64_t)ny * nz * 5 * B;
    const size_t sm = (size_t)(X + 2 * xpad_len<C>(X * nl)) * sizeof(C) + nl * sizeof(XLine);
    const unsigned grid = (unsigned)ceil_div(lines, nl);
    allow_dyn_smem(k_fwd_x<T>, sm);
    k_fwd_x<T><<<grid, kPassThreads, sm, st>>>(x, ldx, p.vmap, L, M, y0, ny, z0, nz, p.nv, lines, A, p.fx, twp[0], nl);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 2 (the register pass over 64-byte row segments by default for complex64: on the 512 x 512
  // and 1024 x 1024 padded grids it ran 25-40 % faster than over 128-byte segments)
  const bool y_narrow = p.y_variant_now == 3 || (p.y_variant_now == 0 && sizeof(C) == 8);
  const bool y_reg =
      p.y_variant_now != 2 &&
      pass_y_reg<-1>(Y, A, ny, ny, Bf, Y, Y, X, (unsigned)(5 * nz * B), twp[1], y0, 0, st, y_narrow);
  if (!y_reg) {
    const int tx = y_lines_per_cta(Y, X, dbl);
    const size_t sm = (size_t)(Y + 2 * Y * tx) * sizeof(C);
    dim3 grid((unsigned)ceil_div(X, tx), (unsigned)(5 * nz * B));
    allow_dyn_smem(k_pass_y<T, -1>, sm);
    k_pass_y<T, -1><<<grid, kPassThreads, sm, st>>>(A, ny, ny, Bf, Y, Y, X, p.fy, twp[1], tx, y0, 0);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 3 (complex64: the real/imaginary tensor when the spectrum has that form)
  bool z_done = false;
  if constexpr (std::is_same<T, float>::value) {
    if (p.z_variant_now == 3) z_done = zpass_toep(p, Bf, B, st);
    if (!z_done && p.tens32ri)
      z_done = zpass_any<float>(p.z_variant_now, Z, nz, Bf, static_cast<const float*>(p.tens32ri), Y, X, B, twp[2], st);
  }
  if constexpr (std::is_same<T, dfloat>::value) {
    if (p.z_variant_now == 3) z_done = zpass_toep_df(p, Bf, B, st);
    if (!z_done) z_done = zpass_df(p.z_variant_now, Z, nz, Bf, static_cast<const dfloat*>(p.tensdf), Y, X, B, twp[2], st);
    VH_REQUIRE(z_done, ERR_UNSUPPORTED, "double-float z-pass length");
  } else if (!z_done && !zpass_any<T>(p.z_variant_now, Z, nz, Bf, tens, Y, X, B, twp[2], st)) {
    const int tx = z_lines_per_cta(Z, X);
    const size_t sm = (size_t)(Z + 2 * Z * 5 * tx) * sizeof(C);
    dim3 grid((unsigned)ceil_div(X, tx), (unsigned)Y);
    allow_dyn_smem(k_zpass<T>, sm);
    k_zpass<T><<<grid, Z * tx, sm, st>>>(Bf, tens, z0, nz, Y, X, B, p.fz, twp[2], tx);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 4
  if (y_reg) {
    pass_y_reg<+1>(Y, Bf, Y, Y, A, ny, ny, X, (unsigned)(5 * nz * B), twp[1], 0, y0, st, y_narrow);
  } else {
    const int tx = y_lines_per_cta(Y, X, dbl);
    const size_t sm = (size_t)(Y + 2 * Y * tx) * sizeof(C);
    dim3 grid((unsigned)ceil_div(X, tx), (unsigned)(5 * nz * B));
    allow_dyn_smem(k_pass_y<T, +1>, sm);
    k_pass_y<T, +1><<<grid, kPassThreads, sm, st>>>(Bf, Y, Y, A, ny, ny, X, p.fy, twp[1], tx, 0, y0);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 5
  if (x_warp) {
    if constexpr (std::is_same<T, float>::value) xpass_warp_inv(p, B, A, x, ldx, y, ldy, scale, zdiag, zstride, st);
  } else {
    const int nl = x_lines_per_cta(X, TileCfg<T>::target);
    const int64_t lines = (int64_t)ny * nz * 5 * B;
    const size_t sm = (size_t)(X + 2 * xpad_len<C>(X * nl)) * sizeof(C) + nl * (sizeof(XLine) + sizeof(float2));
    const unsigned grid = (unsigned)ceil_div(lines, nl);
    allow_dyn_smem(k_inv_x<T>, sm);
    k_inv_x<T><<<grid, kPassThreads, sm, st>>>(A, p.vmap, L, M, y0, ny, z0, nz, p.nv, lines, x, ldx, y, ldy, scale, zdiag,
                                      zstride, 1.0 / p.dx, p.fx, twp[0], nl);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
}

// the complex64 and double-float instantiations (vh_conv_c64.cu, vh_conv_df.cu)
void conv_apply_c64(ConvPlan& p, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy, const double2* scale,
                    const double2* zdiag, int64_t zstride, cudaStream_t st);
void conv_apply_df(ConvPlan& p, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy, const double2* scale,
                   const double2* zdiag, int64_t zstride, cudaStream_t st);

}  // namespace vh
