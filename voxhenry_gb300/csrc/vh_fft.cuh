// Mixed-radix Stockham FFT on lines held in shared memory.
//
// A CTA transforms `nlines` lines of length n at once.  Element i of line l
// lives at buf[i * es + l * ls] (es/ls chosen per pass so that the global
// loads of that pass stay coalesced).  Stages use radices 2, 3, 4, 5, 7 or 8
// (n = 2^a 3^b 5^c 7^d); each stage reads one buffer and writes the other
// (self-sorting Stockham: output in natural order, no digit reversal pass).
//
// Stage with radix R after stages whose radices multiply to Ns:
//   for each butterfly j in [0, n/R):   k = j mod Ns
//     v_r = src[j + r n/R] * w^(r k),  w = exp(DIR 2 pi i / (Ns R))
//     v   = DFT_R(v)
//     dst[(j / Ns) Ns R + k + r Ns] = v_r
// Twiddles come from a table tw[m] = exp(-2 pi i m / n) (conjugated for the
// inverse transform): w^(r k) = tw[r k n / (Ns R)].
#pragma once
#include "vh_common.cuh"

namespace vh {

constexpr int kMaxStages = 24;

struct FftDesc {
  int n;
  int nstages;
  signed char radix[kMaxStages];
};

// ---------------------------------------------------------------- small DFTs
template <int DIR, typename C> __device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int DIR, typename C> __device__ __forceinline__ void dft4(C* v) {
  C t0 = cadd(v[0], v[2]);
  C t1 = csub(v[0], v[2]);
  C t2 = cadd(v[1], v[3]);
  C t3 = cmul_i<DIR>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <int DIR, typename C> __device__ __forceinline__ void dft8(C* v) {
  using T = decltype(v[0].x);
  const T h = (T)0.70710678118654752440084436210484903928483593768847;
  // radix-2 split into even / odd halves
  C a[4] = {v[0], v[2], v[4], v[6]};
  C b[4] = {v[1], v[3], v[5], v[7]};
  dft4<DIR>(a);
  dft4<DIR>(b);
  // twiddles exp(DIR 2 pi i k / 8), k = 0..3
  C b1, b2, b3;
  if (DIR < 0) {
    b1 = mk((b[1].x + b[1].y) * h, (b[1].y - b[1].x) * h);
    b2 = cmul_i<DIR>(b[2]);
    b3 = mk((b[3].y - b[3].x) * h, -(b[3].x + b[3].y) * h);
  } else {
    b1 = mk((b[1].x - b[1].y) * h, (b[1].x + b[1].y) * h);
    b2 = cmul_i<DIR>(b[2]);
    b3 = mk(-(b[3].x + b[3].y) * h, (b[3].x - b[3].y) * h);
  }
  v[0] = cadd(a[0], b[0]);
  v[4] = csub(a[0], b[0]);
  v[1] = cadd(a[1], b1);
  v[5] = csub(a[1], b1);
  v[2] = cadd(a[2], b2);
  v[6] = csub(a[2], b2);
  v[3] = cadd(a[3], b3);
  v[7] = csub(a[3], b3);
}

template <int DIR, typename C> __device__ __forceinline__ void dft3(C* v) {
  using T = decltype(v[0].x);
  const T s3 = (T)0.86602540378443864676372317075293618347140262690519;  // sqrt(3)/2
  C t1 = cadd(v[1], v[2]);
  C t2 = csub(v[1], v[2]);
  C m = mk(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
  // s = DIR * i * sqrt(3)/2 * t2
  C s = cscale(cmul_i<DIR>(t2), s3);
  v[0] = cadd(v[0], t1);
  v[1] = cadd(m, s);
  v[2] = csub(m, s);
}

template <int DIR, typename C> __device__ __forceinline__ void dft5(C* v) {
  using T = decltype(v[0].x);
  const T c1 = (T)0.30901699437494742410229341718281905886436448684462;   // cos(2pi/5)
  const T c2 = (T)-0.80901699437494742410229341718281905886436448684462;  // cos(4pi/5)
  const T s1 = (T)0.95105651629515357211643933337938214340569863412575;   // sin(2pi/5)
  const T s2 = (T)0.58778525229247312916870595463907276859765243764314;   // sin(4pi/5)
  C a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
  C a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
  C m1 = mk(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
  C m2 = mk(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
  // DIR*i*(s1 b1 + s2 b2), DIR*i*(s2 b1 - s1 b2)
  C n1 = cmul_i<DIR>(mk(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
  C n2 = cmul_i<DIR>(mk(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
  v[0] = mk(v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y);
  v[1] = cadd(m1, n1);
  v[4] = csub(m1, n1);
  v[2] = cadd(m2, n2);
  v[3] = csub(m2, n2);
}

template <int DIR, typename C> __device__ __forceinline__ void dft7(C* v) {
  using T = decltype(v[0].x);
  const T c[3] = {(T)0.62348980185873353052500488400423981063227473089640,    // cos(2pi/7)
                  (T)-0.22252093395631440428890256449679475946635556876451,   // cos(4pi/7)
                  (T)-0.90096886790241912623610231950744505116591916213189};  // cos(6pi/7)
  const T s[3] = {(T)0.78183148246802980870844452667405775023233451870868,    // sin(2pi/7)
                  (T)0.97492791218182360701813168299393121723278580062000,    // sin(4pi/7)
                  (T)0.43388373911755812047576833284835875460999072778746};   // sin(6pi/7)
  C a[3], b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a[k] = cadd(v[k + 1], v[6 - k]);
    b[k] = csub(v[k + 1], v[6 - k]);
  }
  C x0 = v[0];
  C out0 = x0;
#pragma unroll
  for (int k = 0; k < 3; ++k) out0 = cadd(out0, a[k]);
#pragma unroll
  for (int m = 1; m <= 3; ++m) {
    C re = x0, im = mk((T)0, (T)0);
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
      int idx = (m * k) % 7;  // angle index
      T cc, ss;
      if (idx <= 3) { cc = c[idx - 1]; ss = s[idx - 1]; } else { cc = c[7 - idx - 1]; ss = -s[7 - idx - 1]; }
      re.x += cc * a[k - 1].x;
      re.y += cc * a[k - 1].y;
      im.x += ss * b[k - 1].x;
      im.y += ss * b[k - 1].y;
    }
    C n = cmul_i<DIR>(im);
    v[m] = cadd(re, n);
    v[7 - m] = csub(re, n);
  }
  v[0] = out0;
}

// ---------------------------------------------------------------- one stage
template <int R, int DIR, typename C>
__device__ __forceinline__ void fft_stage(const C* __restrict__ src, C* __restrict__ dst, const C* __restrict__ tw,
                                          int n, int Ns, int es, int ls, int nlines, bool jfast) {
  const int nb = n / R;
  const int total = nb * nlines;
  const int twmul = n / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int line, j;
    if (jfast) { j = t % nb; line = t / nb; } else { line = t % nlines; j = t / nlines; }
    const int k = j % Ns;
    const int base = line * ls;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[base + (j + r * nb) * es];
    if (Ns > 1) {
      const int step = k * twmul;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = tw[r * step];
        v[r] = (DIR < 0) ? cmul(v[r], w) : cmulc(v[r], w);
      }
    }
    if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
    else if constexpr (R == 3) dft3<DIR>(v);
    else if constexpr (R == 4) dft4<DIR>(v);
    else if constexpr (R == 5) dft5<DIR>(v);
    else if constexpr (R == 7) dft7<DIR>(v);
    else if constexpr (R == 8) dft8<DIR>(v);
    const int d0 = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[base + (d0 + r * Ns) * es] = v[r];
  }
}

// ---- the same stages for a power-of-two length fixed at compile time: the index arithmetic is
// shifts and masks, and the twiddle strides and the radix sequence (radix 8 while it divides, then
// one radix 4 or 2, the order fft_factor gives) are constants.  Every stage does the arithmetic of
// the runtime stage above, so the results are identical.
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

template <int R, int N, int NS, int DIR, typename C>
__device__ __forceinline__ void fft_stage_p2(const C* __restrict__ src, C* __restrict__ dst, const C* __restrict__ tw,
                                             int es, int ls, int nlines, int lognl, bool jfast) {
  constexpr int nb = N / R;
  constexpr int lognb = ilog2c(nb);
  constexpr int logns = ilog2c(NS);
  constexpr int twmul = N / (NS * R);
  const int total = nb * nlines;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int line, j;
    if (jfast) { j = t & (nb - 1); line = t >> lognb; } else { line = t & (nlines - 1); j = t >> lognl; }
    const int k = j & (NS - 1);
    const int base = line * ls;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[base + (j + r * nb) * es];
    if constexpr (NS > 1) {
      const int step = k * twmul;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = tw[r * step];
        v[r] = (DIR < 0) ? cmul(v[r], w) : cmulc(v[r], w);
      }
    }
    if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
    else if constexpr (R == 4) dft4<DIR>(v);
    else dft8<DIR>(v);
    const int d0 = ((j >> logns) << (logns + ilog2c(R))) + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[base + (d0 + r * NS) * es] = v[r];
  }
}

template <int N, int NS, int DIR, typename C>
__device__ __forceinline__ C* fft_stages_p2(C* src, C* dst, const C* tw, int es, int ls, int nlines, int lognl,
                                            bool jfast) {
  if constexpr (NS >= N) {
    return src;
  } else {
    constexpr int rem = N / NS;
    constexpr int R = rem % 8 == 0 ? 8 : (rem % 4 == 0 ? 4 : 2);
    fft_stage_p2<R, N, NS, DIR>(src, dst, tw, es, ls, nlines, lognl, jfast);
    __syncthreads();
    return fft_stages_p2<N, NS * R, DIR>(dst, src, tw, es, ls, nlines, lognl, jfast);
  }
}

// ---- fully static stages: length N, NL lines, layout (JF: line-major, element stride 1 and line
// stride N; else line-interleaved, element stride NL and line stride 1) and NT threads fixed at
// compile time, so each stage is a fixed number of unrolled rounds without bound checks.  The
// arithmetic is that of the stages above.
// PADLOG > 0: the buffers hold logical element a at a + (a >> PADLOG) (one padding element per
// 2^PADLOG), which spreads a stage's strided stores over the banks.
template <int PADLOG>
__device__ __forceinline__ int pad_index(int a) {
  if constexpr (PADLOG > 0) return a + (a >> PADLOG);
  else return a;
}

template <int R, int N, int NS, int NL, bool JF, int DIR, int NT, int PADLOG, typename C>
__device__ __forceinline__ void fft_stage_fixed(const C* __restrict__ src, C* __restrict__ dst, const C* __restrict__ tw) {
  constexpr int nb = N / R;
  constexpr int total = nb * NL;
  constexpr int ES = JF ? 1 : NL, LS = JF ? N : 1;
  constexpr int lognb = ilog2c(nb), lognl = ilog2c(NL), logns = ilog2c(NS);
  constexpr int twmul = N / (NS * R);
  static_assert(JF || (NL & (NL - 1)) == 0, "interleaved lines: power-of-two count");
#pragma unroll
  for (int t0 = 0; t0 < total; t0 += NT) {
    const int t = t0 + (int)threadIdx.x;
    if (total % NT != 0 && t >= total) break;
    int line, j;
    if constexpr (JF) { j = t & (nb - 1); line = t >> lognb; } else { line = t & (NL - 1); j = t >> lognl; }
    const int k = j & (NS - 1);
    const int base = line * LS;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[pad_index<PADLOG>(base + (j + r * nb) * ES)];
    if constexpr (NS > 1) {
      const int step = k * twmul;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = tw[r * step];
        v[r] = (DIR < 0) ? cmul(v[r], w) : cmulc(v[r], w);
      }
    }
    if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
    else if constexpr (R == 4) dft4<DIR>(v);
    else dft8<DIR>(v);
    const int d0 = ((j >> logns) << (logns + ilog2c(R))) + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[pad_index<PADLOG>(base + (d0 + r * NS) * ES)] = v[r];
  }
}

template <int N, int NS, int NL, bool JF, int DIR, int NT, int PADLOG = 0, typename C>
__device__ __forceinline__ C* fft_stages_fixed(C* src, C* dst, const C* tw) {
  if constexpr (NS >= N) {
    return src;
  } else {
    constexpr int rem = N / NS;
    constexpr int R = rem % 8 == 0 ? 8 : (rem % 4 == 0 ? 4 : 2);
    fft_stage_fixed<R, N, NS, NL, JF, DIR, NT, PADLOG>(src, dst, tw);
    __syncthreads();
    return fft_stages_fixed<N, NS * R, NL, JF, DIR, NT, PADLOG>(dst, src, tw);
  }
}

// Runs all stages; returns the buffer holding the result (buf0 or buf1).
// Must be called by all threads of the CTA; ends with a __syncthreads().
template <int DIR, typename C>
__device__ C* fft_lines(C* buf0, C* buf1, const C* tw, const FftDesc& d, int es, int ls, int nlines, bool jfast) {
  // power-of-two lengths 16..2048 (and, for the line-interleaved layout, a power-of-two line
  // count) take the compile-time stages
  if ((d.n & (d.n - 1)) == 0 && d.n >= 16 && d.n <= 2048 && (jfast || (nlines & (nlines - 1)) == 0)) {
    const int lognl = jfast ? 0 : __ffs(nlines) - 1;
    switch (__ffs(d.n) - 1) {
      case 4: return fft_stages_p2<16, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      case 5: return fft_stages_p2<32, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      case 6: return fft_stages_p2<64, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      case 7: return fft_stages_p2<128, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      case 8: return fft_stages_p2<256, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      case 9: return fft_stages_p2<512, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      case 10: return fft_stages_p2<1024, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
      default: return fft_stages_p2<2048, 1, DIR>(buf0, buf1, tw, es, ls, nlines, lognl, jfast);
    }
  }
  C* src = buf0;
  C* dst = buf1;
  int Ns = 1;
  for (int s = 0; s < d.nstages; ++s) {
    const int R = d.radix[s];
    switch (R) {
      case 2: fft_stage<2, DIR>(src, dst, tw, d.n, Ns, es, ls, nlines, jfast); break;
      case 3: fft_stage<3, DIR>(src, dst, tw, d.n, Ns, es, ls, nlines, jfast); break;
      case 4: fft_stage<4, DIR>(src, dst, tw, d.n, Ns, es, ls, nlines, jfast); break;
      case 5: fft_stage<5, DIR>(src, dst, tw, d.n, Ns, es, ls, nlines, jfast); break;
      case 7: fft_stage<7, DIR>(src, dst, tw, d.n, Ns, es, ls, nlines, jfast); break;
      default: fft_stage<8, DIR>(src, dst, tw, d.n, Ns, es, ls, nlines, jfast); break;
    }
    __syncthreads();
    C* t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  return src;
}

// ---- register-resident pruned transforms of a compile-time power-of-two length (one line per
// thread).  tw[j] = exp(-2 pi i j / Z) for the top-level length Z; DIR = -1 forward, +1 inverse
// (unnormalised).  Multiplications by 1, -+i and exp(-+i pi/4) are resolved at compile time.
template <int Z, int N, int DIR, typename C>
__host__ __device__ __forceinline__ C tw_mul(C x, int n, const C* tw) {
  if (n == 0) return x;
  if (4 * n == N) return cmul_i<DIR>(x);
  const C w = tw[n * (Z / N)];
  if (8 * n == N) {   // w = (c, -+c), c = cos(pi/4)
    const auto c = w.x;
    C r;
    if (DIR < 0) { r.x = (x.x + x.y) * c; r.y = (x.y - x.x) * c; }
    else { r.x = (x.x - x.y) * c; r.y = (x.x + x.y) * c; }
    return r;
  }
  return DIR < 0 ? cmul(x, w) : cmulc(x, w);
}

// Decimation in frequency, natural-order input whose entries at or beyond NZ are zero (they are
// not read), bit-reversed output.  A half whose upper part is zero costs only its twiddles.
template <int Z, int N, int NZ, int DIR, typename C>
__host__ __device__ __forceinline__ void dif_pruned(C* v, const C* tw) {
  if constexpr (N > 1) {
    constexpr int H = N / 2;
#pragma unroll
    for (int n = 0; n < H; ++n) {
      if (n >= NZ) continue;                       // both zero
      if (n + H >= NZ) {                           // upper zero
        v[n + H] = tw_mul<Z, N, DIR>(v[n], n, tw);
      } else {
        const C a = v[n], b = v[n + H];
        v[n] = cadd(a, b);
        v[n + H] = tw_mul<Z, N, DIR>(csub(a, b), n, tw);
      }
    }
    constexpr int NZ2 = NZ < H ? NZ : H;
    dif_pruned<Z, H, NZ2, DIR>(v, tw);
    dif_pruned<Z, H, NZ2, DIR>(v + H, tw);
  }
}

// Decimation in time, bit-reversed input, natural-order output of which only entries below NZ
// are formed.
template <int Z, int N, int NZ, int DIR, typename C>
__host__ __device__ __forceinline__ void dit_pruned(C* v, const C* tw) {
  if constexpr (N > 1) {
    constexpr int H = N / 2;
    constexpr int NZ2 = NZ < H ? NZ : H;
    dit_pruned<Z, H, NZ2, DIR>(v, tw);
    dit_pruned<Z, H, NZ2, DIR>(v + H, tw);
#pragma unroll
    for (int k = 0; k < H; ++k) {
      const bool lo = k < NZ, hi = k + H < NZ;
      if (!lo && !hi) continue;
      const C t = tw_mul<Z, N, DIR>(v[k + H], k, tw);
      if (hi) v[k + H] = csub(v[k], t);
      if (lo) v[k] = cadd(v[k], t);
    }
  }
}

template <int BITS>
__host__ __device__ constexpr int bit_reverse(int x) {
  int r = 0;
  for (int b = 0; b < BITS; ++b) r |= ((x >> b) & 1) << (BITS - 1 - b);
  return r;
}

}  // namespace vh
