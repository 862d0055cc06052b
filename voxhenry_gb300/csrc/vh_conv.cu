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
#include <vector>

#include "vh_conv.cuh"
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

// ------------------------------------------------------------------------------------------
template <typename T> struct TileCfg;
template <> struct TileCfg<double> { static constexpr int target = 2048; };
template <> struct TileCfg<float> { static constexpr int target = 2048; };

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

template <int DIR, typename C>
__device__ __forceinline__ C* fft_x_lines(C* b0, C* b1, const C* tw, const FftDesc& fd, int nl) {
  if (blockDim.x == kPassThreads) {
    if (fd.n == 256 && nl == 8) return fft_stages_fixed<256, 1, 8, true, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 512 && nl == 4) return fft_stages_fixed<512, 1, 4, true, DIR, kPassThreads>(b0, b1, tw);
    if (fd.n == 1024 && nl == 2) return fft_stages_fixed<1024, 1, 2, true, DIR, kPassThreads>(b0, b1, tw);
  }
  return fft_lines<DIR>(b0, b1, tw, fd, 1, fd.n, nl, true);
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
  return fft_lines<DIR>(b0, b1, tw, fd, tx, 1, tx, false);
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
  C* b1 = b0 + X * nl;
  XLine* li = reinterpret_cast<XLine*>(b1 + X * nl);
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
    b0[line * X + L + (t - line * XL)] = czero<C>();
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
        b0[line * X + (t - line * L)] = v;
      }
    }
  }
  __syncthreads();
  C* r = fft_x_lines<-1>(b0, b1, tw, fd, nl);
  const int rows = (nlines_total - l0 < nl) ? (int)(nlines_total - l0) : nl;
  tile_store(A + l0 * X, X, r, X, rows, X);
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

// pass 3 for Z = 8, 16, 32: one thread transforms one column of one component in registers.  The
// nz voxel rows enter the transform at rows 0.. (circular convolution is shift invariant), so the
// forward transform reads only NZ >= nz leading rows and the inverse forms only the first NZ rows
// (pruned at compile time).  Block: 5 warps (warp = component, lane = kx column) over 32 columns of
// one ky row; the five spectra of a point meet in shared memory for the tensor product.
constexpr int kZregCols = 32;

// storage <-> arithmetic type of the z-pass (identity, or complex128 storage with double-float
// arithmetic)
__device__ __forceinline__ float2 zload(float2 v, float2) { return v; }
__device__ __forceinline__ double2 zload(double2 v, double2) { return v; }
__device__ __forceinline__ dcomplex zload(double2 v, dcomplex) { return to_c(v, dcomplex()); }
__device__ __forceinline__ float2 zstore(float2 v, float2) { return v; }
__device__ __forceinline__ double2 zstore(double2 v, double2) { return v; }
__device__ __forceinline__ double2 zstore(dcomplex v, double2) { return to_d(v); }

template <typename T, int Z, int NZ, typename ST = cplx<T>, typename GT = cplx<T>>
__global__ void __launch_bounds__(5 * kZregCols)
    k_zpass_reg(ST* __restrict__ Bf, const GT* __restrict__ tens, int nz, int Y, int X, int nrhs,
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
  const int kx = blockIdx.x * kZregCols + lane;
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
      for (int p = 0; p < Z; ++p) S[(warp * Z + p) * kZregCols + lane] = v[p];
    }
    __syncthreads();
    if constexpr (kHoist) {
#pragma unroll
      for (int qi = 0; qi < Q; ++qi) {
        const int p = warp + 5 * qi;
        if (p < Z) {
          C* q = S + p * kZregCols + lane;
          constexpr int cs = Z * kZregCols;
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
        C* q = S + p * kZregCols + lane;
        constexpr int cs = Z * kZregCols;
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
      for (int p = 0; p < Z; ++p) v[p] = S[(warp * Z + p) * kZregCols + lane];
      dit_pruned<Z, Z, NZ, +1>(v, tw);
#pragma unroll
      for (int i = 0; i < NZ; ++i)
        if (i < nz && col_ok) base[warp * comp + i * plane] = zstore(v[i], ST());
    }
    __syncthreads();   // S is rewritten by the next RHS
  }
}

template <typename T, int Z, int NZ, typename ST, typename GT>
static void launch_zpass_reg(ST* Bf, const GT* tens, int nz, int Y, int X, int B, const cplx<T>* tw,
                             cudaStream_t st) {
  const size_t sm = (size_t)(Z + 5 * Z * kZregCols) * sizeof(cplx<T>);
  VH_CUDA_TRY(cudaFuncSetAttribute(k_zpass_reg<T, Z, NZ, ST, GT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sm));
  dim3 grid((unsigned)ceil_div(X, kZregCols), (unsigned)Y);
  k_zpass_reg<T, Z, NZ, ST, GT><<<grid, 5 * kZregCols, sm, st>>>(Bf, tens, nz, Y, X, B, tw);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

// true when the register z-pass handles this length (Z = 8, 16, 32; nz <= Z / 2 always holds);
// T is the arithmetic type, ST the storage type of the spectra
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
    default: return false;
  }
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
  C* b1 = b0 + X * nl;
  XLine* li = reinterpret_cast<XLine*>(b1 + X * nl);
  for (int i = threadIdx.x; i < X; i += blockDim.x) tw[i] = twg[i];
  const int64_t l0 = (int64_t)blockIdx.x * nl;
  const int rows_valid = (nlines_total - l0 < nl) ? (int)(nlines_total - l0) : nl;
  float2* sline = reinterpret_cast<float2*>(li + nl);   // the line's RHS scale in FP32 (complex64 product)
  decode_lines(li, l0, nl, nlines_total, L, M, y0, ny, z0, nz, ldx, nv);
  if constexpr (sizeof(T) == 4) {
    for (int line = threadIdx.x; line < nl; line += blockDim.x) sline[line] = to_c(scale[li[line].b], float2());
  }
  tile_load(b0, X, A + l0 * X, X, nl, rows_valid, X, X);
  cp_async_wait_all();
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
      const float2 conv = r[line * X + i];
      const float2 sf = sline[line], zf = to_c(zz, float2()), xf = to_c(xj, float2());
      const float2 d = cmul(zf, xf);
      const float ckf = (float)ck;
      float2 o = cmul(sf, conv);
      o.x = fmaf(ckf, d.x, o.x);
      o.y = fmaf(ckf, d.y, o.y);
      yout[b * ldy + c * nv + vid] = make_double2((double)o.x, (double)o.y);
    } else {
      const double2 conv = to_d(r[line * X + i]);
      double2 out = cmul(scale[b], conv);
      out = cadd(out, cscale(cmul(zz, xj), ck));
      yout[b * ldy + c * nv + vid] = out;
    }
  }
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
  if (want32) {
    VH_CUDA_TRY(cudaMalloc(&p.tens32, 7 * P * sizeof(float2)));
    k_tensor_permute<float2><<<1024, 256, 0, st>>>(fN_all_dev, p.tens32, p.X, p.Y, p.Z, s);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    // real/imaginary check of each component over the whole spectrum
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
    if (ri) {
      VH_CUDA_TRY(cudaMalloc(&p.tens32ri, 7 * P * sizeof(float)));
      k_tensor_permute_ri<<<1024, 256, 0, st>>>(fN_all_dev, p.tens32ri, p.X, p.Y, p.Z, s);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    }
  }
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

// the double-float tensor spectrum and z twiddles for PREC_DF, from tens64 (once per plan)
__global__ void k_tensor_to_df(const double2* __restrict__ in, dcomplex* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = to_c(in[i], dcomplex());
}

static void ensure_df_tensor(ConvPlan& p, cudaStream_t st) {
  if (p.tensdf) return;
  const int64_t n = 7 * p.points();
  VH_CUDA_TRY(cudaMalloc(&p.tensdf, n * sizeof(dcomplex)));
  k_tensor_to_df<<<1024, 256, 0, st>>>(p.tens64, static_cast<dcomplex*>(p.tensdf), n);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
  const auto t = twiddles(p.Z);
  std::vector<dcomplex> td(p.Z);
  for (int i = 0; i < p.Z; ++i) td[i] = dcomplex{dfloat(t[i].x), dfloat(t[i].y)};
  VH_CUDA_TRY(cudaMalloc(&p.twdf, p.Z * sizeof(dcomplex)));
  VH_CUDA_TRY(cudaMemcpyAsync(p.twdf, td.data(), p.Z * sizeof(dcomplex), cudaMemcpyHostToDevice, st));
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

void conv_plan_destroy(ConvPlan& p) {
  cudaFree(p.vmap);
  cudaFree(p.tens64);
  cudaFree(p.tens32);
  cudaFree(p.tens32ri);
  cudaFree(p.tensdf);
  cudaFree(p.twdf);
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

template <typename T>
static void conv_apply_t(ConvPlan& p, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                         const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st,
                         bool df_z = false) {
  using C = cplx<T>;
  const bool dbl = sizeof(T) == 8;
  C* A = reinterpret_cast<C*>(p.scratchA);
  C* Bf = reinterpret_cast<C*>(p.scratchB);
  const C* tens = dbl ? reinterpret_cast<const C*>(p.tens64) : reinterpret_cast<const C*>(p.tens32);
  C* const* twp = dbl ? reinterpret_cast<C* const*>(p.tw64) : reinterpret_cast<C* const*>(p.tw32);
  VH_REQUIRE(tens != nullptr, ERR_BAD_ARG, "tensor for this precision was not built");
  const int X = p.X, Y = p.Y, Z = p.Z, L = p.L, M = p.M;
  const int y0 = p.y0, ny = p.ny, z0 = p.z0, nz = p.nz;
  VH_REQUIRE(ny > 0 && nz > 0, ERR_BAD_ARG, "FFT convolution of a geometry without voxels");
  // pass 1
  {
    const int nl = x_lines_per_cta(X, TileCfg<T>::target);
    const int64_t lines = (int64_t)ny * nz * 5 * B;
    const size_t sm = (size_t)(X + 2 * X * nl) * sizeof(C) + nl * sizeof(XLine);
    const unsigned grid = (unsigned)ceil_div(lines, nl);
    VH_CUDA_TRY(cudaFuncSetAttribute(k_fwd_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_fwd_x<T><<<grid, kPassThreads, sm, st>>>(x, ldx, p.vmap, L, M, y0, ny, z0, nz, p.nv, lines, A, p.fx, twp[0], nl);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 2
  {
    const int tx = y_lines_per_cta(Y, X, dbl);
    const size_t sm = (size_t)(Y + 2 * Y * tx) * sizeof(C);
    dim3 grid((unsigned)ceil_div(X, tx), (unsigned)(5 * nz * B));
    VH_CUDA_TRY(cudaFuncSetAttribute(k_pass_y<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_pass_y<T, -1><<<grid, kPassThreads, sm, st>>>(A, ny, ny, Bf, Y, Y, X, p.fy, twp[1], tx, y0, 0);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 3 (double-float arithmetic on the complex128 spectra when asked and the length allows)
  bool z_done = false;
  if constexpr (sizeof(T) == 8) {
    if (df_z && p.tensdf)
      z_done = zpass_reg<dfloat>(Z, nz, Bf, static_cast<const dcomplex*>(p.tensdf), Y, X, B,
                                 static_cast<const dcomplex*>(p.twdf), st);
  }
  if constexpr (sizeof(T) == 4) {
    if (p.tens32ri) z_done = zpass_reg<float>(Z, nz, Bf, static_cast<const float*>(p.tens32ri), Y, X, B, twp[2], st);
  }
  if (!z_done && !zpass_reg<T>(Z, nz, Bf, tens, Y, X, B, twp[2], st)) {
    const int tx = z_lines_per_cta(Z, X);
    const size_t sm = (size_t)(Z + 2 * Z * 5 * tx) * sizeof(C);
    dim3 grid((unsigned)ceil_div(X, tx), (unsigned)Y);
    VH_CUDA_TRY(cudaFuncSetAttribute(k_zpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_zpass<T><<<grid, Z * tx, sm, st>>>(Bf, tens, z0, nz, Y, X, B, p.fz, twp[2], tx);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 4
  {
    const int tx = y_lines_per_cta(Y, X, dbl);
    const size_t sm = (size_t)(Y + 2 * Y * tx) * sizeof(C);
    dim3 grid((unsigned)ceil_div(X, tx), (unsigned)(5 * nz * B));
    VH_CUDA_TRY(cudaFuncSetAttribute(k_pass_y<T, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_pass_y<T, +1><<<grid, kPassThreads, sm, st>>>(Bf, Y, Y, A, ny, ny, X, p.fy, twp[1], tx, 0, y0);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  // pass 5
  {
    const int nl = x_lines_per_cta(X, TileCfg<T>::target);
    const int64_t lines = (int64_t)ny * nz * 5 * B;
    const size_t sm = (size_t)(X + 2 * X * nl) * sizeof(C) + nl * (sizeof(XLine) + sizeof(float2));
    const unsigned grid = (unsigned)ceil_div(lines, nl);
    VH_CUDA_TRY(cudaFuncSetAttribute(k_inv_x<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_inv_x<T><<<grid, kPassThreads, sm, st>>>(A, p.vmap, L, M, y0, ny, z0, nz, p.nv, lines, x, ldx, y, ldy, scale, zdiag,
                                      zstride, 1.0 / p.dx, p.fx, twp[0], nl);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
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
    VH_CUDA_TRY(cudaFuncSetAttribute(k_fft_axis_inplace, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
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
  conv_plan_reserve(p, B, prec);
  if (prec == PREC_DF) ensure_df_tensor(p, st);
  if (prec == PREC_FP32)
    conv_apply_t<float>(p, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
  else
    conv_apply_t<double>(p, B, x, ldx, y, ldy, scale, zdiag, zstride, st, prec == PREC_DF);
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
  q.scratchA = scratchA;
  q.scratchB = scratchB;
  q.scratch_bytes_A = a1 * B;
  q.scratch_bytes_B = b1 * B;
  if (prec == PREC_FP32)
    conv_apply_t<float>(q, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
  else   // PREC_DF uses the double-float z-pass only if the plan already holds its tensor
    conv_apply_t<double>(q, B, x, ldx, y, ldy, scale, zdiag, zstride, st, prec == PREC_DF);
}

}  // namespace vh
