// Multifrontal Cholesky of S = Ar D Ar^T on the device: numeric factorisation and solves.
//
// Factor storage W: one dense nf x nf column-major block per front.  After the factorisation
// its first ns columns hold [L11; L21] (with each 32 x 32 diagonal block of L11 replaced by its
// inverse) and its trailing nb x nb block holds the update matrix passed to the parent
// (extend-add).  All fronts of one tree height are processed together; heights run from the
// leaves up.  Fronts with nf <= kFusedMaxNf are factored whole in shared memory by one CTA
// (k_chol_front); larger ones by blocks of 32 columns -- diagonal block (one CTA), panel
// (row chunks), symmetric rank-32 update of the trailing lower triangle (64 x 64 tiles).
//
// The kernels are templates on the factor's element type T: double (the reference's arithmetic)
// or dfloat, the FP32-pair format of the mixed-precision solver's factor (about 48 significant
// bits on the FP32 pipes, which GB300 runs at 64 times its FP64 rate).  A plain single-precision
// factor was measured and rejected: on the 256 x 256 x 8 spiral the Schur complement is too
// ill-conditioned (FP32 Cholesky breaks down, and an FP32 LU preconditioner raises GMRES iterations
// from 3-28 to 7-80+).
#include <vector>

#include <type_traits>

#include "vh_chol.cuh"
#include "vh_df.cuh"

namespace vh {

constexpr int kNB = 32;   // panel width
constexpr int kTS = 64;   // update tile

template <typename T> __device__ __forceinline__ T rsqrt_t(T p);
template <> __device__ __forceinline__ double rsqrt_t<double>(double p) { return 1.0 / sqrt(p); }
template <> __device__ __forceinline__ float rsqrt_t<float>(float p) { return 1.0f / sqrtf(p); }
template <> __device__ __forceinline__ dfloat rsqrt_t<dfloat>(dfloat p) { return df_rsqrt(p); }

// ---- assembly of the original entries of S: F(li, lj) = sum_t c_t D(q_t)
// Every factorisation kernel handles gridDim.z factors at once (one per frequency): factor z
// lives at Wp[z] and is built from the diagonal Dp[z].
template <typename T>
__global__ void k_chol_assemble(const FrontInfo* __restrict__ fr, const AsmEntry* __restrict__ ae,
                                const int32_t* __restrict__ aq, const double* __restrict__ ac,
                                const double* const* __restrict__ Dp, T* const* __restrict__ Wp) {
  const FrontInfo f = fr[blockIdx.x];
  const double* D = Dp[blockIdx.z];
  T* F = Wp[blockIdx.z] + f.w_off;
  for (int e = threadIdx.x; e < f.asm_cnt; e += blockDim.x) {
    const AsmEntry a = ae[f.asm_off + e];
    double s = 0.0;
    for (int t = a.t0; t < a.t1; ++t) s = fma(ac[t], D[aq[t]], s);
    F[a.li + (int64_t)a.lj * f.nf] = (T)s;
  }
}

// ---- extend-add of child `which` of every front in the level list
template <typename T>
__global__ void k_chol_extend_add(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                                  const int32_t* __restrict__ relmap, T* const* __restrict__ Wp, int which) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  T* W = Wp[blockIdx.z];
  const int ci = f.child[which];
  if (ci < 0) return;
  const FrontInfo c = fr[ci];
  const int nb = c.nb;
  const int32_t* rm = relmap + c.relmap_off;
  const T* U = W + c.w_off + c.ns + (int64_t)c.ns * c.nf;   // U(a, b) = U[a + b * c.nf]
  T* F = W + f.w_off;
  for (int b = blockIdx.y; b < nb; b += gridDim.y) {
    const int lj = rm[b];
    for (int a = b + threadIdx.x; a < nb; a += blockDim.x) F[rm[a] + (int64_t)lj * f.nf] += U[a + (int64_t)b * c.nf];
  }
}

// ---- Cholesky of the diagonal block [k0, k0+w); the block is replaced by the inverse of its factor
template <typename T>
__global__ void k_chol_diag(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                            T* const* __restrict__ Wp, int k0, int* __restrict__ err) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  T* W = Wp[blockIdx.z];
  if (f.ns <= k0) return;
  const int w = min(kNB, f.ns - k0);
  __shared__ T A[kNB][kNB + 1];
  T* F = W + f.w_off;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int i = t % w, j = t / w;
    A[i][j] = (i >= j) ? F[(k0 + i) + (int64_t)(k0 + j) * f.nf] : T(0);
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const T piv = A[j][j];
    if (!(piv > T(0))) {
      if (threadIdx.x == 0) atomicExch(err, 1);
      return;                                   // uniform across the CTA: piv read after a barrier
    }
    const T inv = rsqrt_t(piv);
    __syncthreads();
    if (threadIdx.x == 0) A[j][j] = piv * inv;
    for (int i = j + 1 + threadIdx.x; i < w; i += blockDim.x) A[i][j] *= inv;
    __syncthreads();
    for (int t = threadIdx.x; t < (w - j - 1) * (w - j - 1); t += blockDim.x) {
      const int i = j + 1 + t % (w - j - 1), k = j + 1 + t / (w - j - 1);
      if (i >= k) A[i][k] -= A[i][j] * A[k][j];
    }
    __syncthreads();
  }
  // Invert the factored block (lower triangular) and store the INVERSE in place of the block:
  // the panel solve and both triangular solves then multiply by it.  Thread j computes column
  // j: Linv(j,j) = 1/A(j,j), Linv(i,j) = -(sum_{k=j}^{i-1} A(i,k) Linv(k,j)) / A(i,i).
  __shared__ T Iv[kNB][kNB + 1];
  if (threadIdx.x < w) {
    const int j = threadIdx.x;
    Iv[j][j] = T(1) / A[j][j];
    for (int i = j + 1; i < w; ++i) {
      T s = T(0);
      for (int k = j; k < i; ++k) s = fma(A[i][k], Iv[k][j], s);
      Iv[i][j] = -s / A[i][i];
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int i = t % w, j = t / w;
    if (i >= j) F[(k0 + i) + (int64_t)(k0 + j) * f.nf] = Iv[i][j];
  }
}

// ---- panel rows [k0+w, nf): L(r, k0:k0+w) = F(r, k0:k0+w) L11^-T
template <typename T>
__global__ void k_chol_panel(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                             T* const* __restrict__ Wp, int k0) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  T* W = Wp[blockIdx.z];
  if (f.ns <= k0) return;
  const int w = min(kNB, f.ns - k0);
  const int r = k0 + w + blockIdx.y * blockDim.x + threadIdx.x;
  __shared__ T A[kNB][kNB + 1];
  T* F = W + f.w_off;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int i = t % w, j = t / w;
    A[i][j] = (i >= j) ? F[(k0 + i) + (int64_t)(k0 + j) * f.nf] : T(0);
  }
  __syncthreads();
  if (r >= f.nf) return;
  // the diagonal block holds L11^-1 (k_chol_diag): L(r, k0+j) = sum_{k <= j} F(r, k0+k) Linv(j, k)
  T a[kNB], x[kNB];
#pragma unroll
  for (int j = 0; j < kNB; ++j) a[j] = j < w ? F[r + (int64_t)(k0 + j) * f.nf] : T(0);
#pragma unroll
  for (int j = 0; j < kNB; ++j) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < kNB; ++k)
      if (k <= j) s = fma(a[k], A[j][k], s);
    x[j] = s;
  }
#pragma unroll
  for (int j = 0; j < kNB; ++j)
    if (j < w) F[r + (int64_t)(k0 + j) * f.nf] = x[j];
}

// ---- trailing update F(r, c) -= sum_k L(r, k) L(c, k) for t0 <= c <= r < nf, k in [k0, k0+w)
template <typename T>
__global__ void __launch_bounds__(256) k_chol_update(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr,
                                                     T* const* __restrict__ Wp, int k0) {
  const FrontInfo f = fr[lev[blockIdx.x]];
  T* W = Wp[blockIdx.z];
  if (f.ns <= k0) return;
  const int w = min(kNB, f.ns - k0);
  const int t0 = k0 + w;
  const int m = f.nf - t0;
  if (m <= 0) return;
  const int nt = (m + kTS - 1) / kTS;
  const int tile = blockIdx.y;
  if (tile >= nt * (nt + 1) / 2) return;
  // tile -> (ti, tj), ti >= tj, row-major over the lower triangle
  int ti = (int)((sqrt(8.0 * tile + 1.0) - 1.0) * 0.5);
  while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
  while (ti * (ti + 1) / 2 > tile) --ti;
  const int tj = tile - ti * (ti + 1) / 2;
  const int r0 = t0 + ti * kTS, c0 = t0 + tj * kTS;
  __shared__ T Pr[kNB][kTS + 1];
  __shared__ T Pc[kNB][kTS + 1];
  T* F = W + f.w_off;
  for (int t = threadIdx.x; t < kNB * kTS; t += blockDim.x) {
    const int i = t % kTS, k = t / kTS;
    const int r = r0 + i, c = c0 + i;
    Pr[k][i] = (k < w && r < f.nf) ? F[r + (int64_t)(k0 + k) * f.nf] : T(0);
    Pc[k][i] = (k < w && c < f.nf) ? F[c + (int64_t)(k0 + k) * f.nf] : T(0);
  }
  __syncthreads();
  const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;   // 4x4 register block per thread
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);
  for (int k = 0; k < w; ++k) {
    T ra[4], cb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) ra[a] = Pr[k][tr + 16 * a];
#pragma unroll
    for (int b = 0; b < 4; ++b) cb[b] = Pc[k][tc + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = fma(ra[a], cb[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int r = r0 + tr + 16 * a, c = c0 + tc + 16 * b;
      if (r < f.nf && c < f.nf && r >= c) F[r + (int64_t)c * f.nf] -= acc[a][b];
    }
}

// ---- whole-front factorisation in shared memory (fronts with nf <= kFusedMaxNf), one CTA of NT
// threads per (front, factor); NT grows with the front (a single warp up to nf = 64, so that small
// fronts are not dominated by per-column overhead).  The front's lower triangle is held packed:
// column k at tri_off(k, nf) - k, rows k..nf-1.  The CTA adds the children's update matrices and
// factors the first ns columns right-looking with one barrier per column: every thread takes the
// square root and reciprocal of the pivot itself, updates the trailing triangle with the unscaled
// column times 1/pivot (walked as one flat index range, every thread busy), and scales the
// previous column, which no thread reads any more, in the same step.  It then writes [L11; L21],
// the update matrix and the inverses of the 32 x 32 diagonal blocks of L11 (the form the
// triangular solves use) back to the factor storage.

// offset of column c in the column-major lower triangle of order m (column c holds m - c entries)
__host__ __device__ __forceinline__ int tri_off(int c, int m) { return c * m - (c * (c - 1)) / 2; }

constexpr int kLoadBatch = 4;   // independent global loads per thread per step of the load phases
constexpr int kPanel = 4;       // pivots per panel of the fused front factorisation

// a / d for 0 <= a < 2^24 and d >= 1, given rd = 1/d rounded to a float: the float estimate is
// within one of the quotient (|a rd - a/d| < a/d * 2^-23), and the integer check corrects it
__device__ __forceinline__ int div_small(int a, int d, float rd) {
  int q = (int)((float)a * rd);
  if (q * d > a) --q;
  else if ((q + 1) * d <= a) ++q;
  return q;
}

template <int NT>
__device__ __forceinline__ void front_bar() {
  if constexpr (NT == 32)
    __syncwarp();
  else
    __syncthreads();
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT)
    k_chol_front(const int32_t* __restrict__ lev, const FrontInfo* __restrict__ fr, const int32_t* __restrict__ relmap,
                 T* const* __restrict__ Wp, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char fused_raw[];
  T* S = reinterpret_cast<T*>(fused_raw);
  const FrontInfo f = fr[lev[blockIdx.x]];
  T* W = Wp[blockIdx.z];
  const int nf = f.nf, ns = f.ns;
  T* F = W + f.w_off;
  T* inv_s = S + nf * (nf + 1) / 2;   // 1 / L(j, j)
  T* coefs = inv_s + ns;                // per panel pivot q: S(j+q+1+c, j+q) / S(j+q, j+q) at coefs[q * nf + c]
  auto col = [&](int k) { return S + tri_off(k, nf) - k; };   // col(k)[i] = (i, k), i >= k
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nwarps = NT / 32;
  // Loads walk flat index ranges with kLoadBatch independent global loads per thread before any
  // shared-memory write (a column-by-column walk leaves one load in flight per thread).
  {
    const int nn = nf * nf;   // column-major nf x nf storage; the lower triangle is kept
    const float rnf = __frcp_rn((float)nf);
    for (int base = tid; base < nn; base += kLoadBatch * NT) {
      T v[kLoadBatch];
      int off[kLoadBatch];
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int idx = base + u * NT;
        off[u] = -1;
        if (idx < nn) {
          const int k = div_small(idx, nf, rnf), i = idx - k * nf;
          if (i >= k) {
            off[u] = tri_off(k, nf) - k + i;
            v[u] = F[idx];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u)
        if (off[u] >= 0) S[off[u]] = v[u];
    }
  }
  front_bar<NT>();
  int32_t* rms = reinterpret_cast<int32_t*>(coefs);   // a child's relative map (nb <= nf entries)
  for (int c = 0; c < 2; ++c) {
    const int ci = f.child[c];
    if (ci < 0) continue;
    const FrontInfo ch = fr[ci];
    const int nb = ch.nb;
    const int32_t* rm = relmap + ch.relmap_off;
    const T* U = W + ch.w_off + ch.ns + (int64_t)ch.ns * ch.nf;   // U(a, b) = U[a + b * ch.nf]
    for (int a = tid; a < nb; a += NT) rms[a] = rm[a];
    front_bar<NT>();
    const int nn = nb * nb;
    const float rnb = __frcp_rn((float)max(nb, 1));
    for (int base = tid; base < nn; base += kLoadBatch * NT) {
      T v[kLoadBatch];
      int off[kLoadBatch];
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u) {
        const int idx = base + u * NT;
        off[u] = -1;
        if (idx < nn) {
          const int b = div_small(idx, nb, rnb), a = idx - b * nb;
          if (a >= b) {
            const int rb = rms[b];
            off[u] = tri_off(rb, nf) - rb + rms[a];
            v[u] = U[a + (int64_t)b * ch.nf];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kLoadBatch; ++u)
        if (off[u] >= 0) S[off[u]] += v[u];
    }
    front_bar<NT>();
  }
  // Pivots go in panels of up to kPanel (j .. j+P-1): each pivot in turn gives its column
  // coefficients and a rank-1 update of the panel's later columns; then one walk over the remaining
  // triangle applies all P pivots to each entry with one load, one pair-precision dot (P products,
  // one normalisation) and one store.  Pivot columns are scaled by 1 / L(j, j) after their last use
  // (deferred to the next panel).
  using Dot = typename dot_of<T>::type;
  int ndef = 0, defj[kPanel];
  T defpiv[kPanel], definv[kPanel];
  auto scale_deferred = [&]() {
    for (int d = 0; d < ndef; ++d) {
      T* colp = col(defj[d]);
      for (int i = defj[d] + tid; i < nf; i += NT) colp[i] = (i == defj[d]) ? defpiv[d] * definv[d] : colp[i] * definv[d];
    }
    ndef = 0;
  };
  // position (c, p) of flat index t in the column-major lower triangle of order m
  auto locate = [&](int t, int m, int& c, int& p) {
    const float mf = 2.0f * m + 1.0f;
    c = (int)((mf - sqrtf(fmaxf(mf * mf - 8.0f * t, 0.0f))) * 0.5f);
    c = max(0, min(c, m - 1));
    while (c > 0 && tri_off(c, m) > t) --c;
    while (c + 1 < m && tri_off(c + 1, m) <= t) ++c;
    p = t - tri_off(c, m);
  };
  for (int j = 0; j < ns;) {
    const int P = min(kPanel, ns - j);
    scale_deferred();
    for (int q = 0; q < P; ++q) {
      const int jq = j + q;
      T* cq = col(jq);
      const T pv = cq[jq];        // final: updated last before the preceding barrier
      if (!(pv > T(0))) {         // uniform: every thread reads the same value
        if (tid == 0) atomicExch(err, 1);
        return;
      }
      const T iv = rsqrt_t(pv);
      const T iv2 = iv * iv;
      if (tid == 0) inv_s[jq] = iv;
      defj[q] = jq;
      defpiv[q] = pv;
      definv[q] = iv;
      T* cf = coefs + q * nf;
      for (int c = tid; c < nf - jq - 1; c += NT) cf[c] = cq[jq + 1 + c] * iv2;   // once per column
      front_bar<NT>();
      const int nk = P - q - 1;   // the panel's later columns jq+1 .. j+P-1 take this pivot now
      if (nk > 0) {
        for (int kk = 0; kk < nk; ++kk) {   // column by column, rows k.. only (no index division)
          const int k = jq + 1 + kk;
          T* ck = col(k);
          const T cfk = cf[kk];
          for (int i = k + tid; i < nf; i += NT) ck[i] = fma(-cq[i], cfk, ck[i]);
        }
        front_bar<NT>();
      }
    }
    ndef = P;
    // S(i, k) -= sum_q S(i, j+q) S(k, j+q) / S(j+q, j+q) for j+P <= k <= i < nf
    const int m = nf - j - P;
    const int total = (m * (m + 1)) / 2;
    if (tid < total) {
      int c, p;
      locate(tid, m, c, p);
      const int k0 = j + P + c;
      T* colk = col(k0) + k0;   // entry (k, k) of column k
      const T* l[kPanel];
      T cfv[kPanel];
#pragma unroll
      for (int q = 0; q < kPanel; ++q) {
        l[q] = col(j + min(q, P - 1)) + k0;   // S(k, j+q)
        cfv[q] = q < P ? coefs[q * nf + c + P - q - 1] : T(0);
      }
      for (;;) {
        Dot acc(colk[p]);
#pragma unroll
        for (int q = 0; q < kPanel; ++q)
          if (q < P) acc.add(-l[q][p], cfv[q]);
        colk[p] = acc.value();
        p += NT;
        if (p >= m - c) {
          do {                    // next column: col(k + 1) + k + 1 = col(k) + k + (nf - k)
            p -= m - c;
            colk += m - c;
#pragma unroll
            for (int q = 0; q < kPanel; ++q) ++l[q];
            ++c;
          } while (c < m && p >= m - c);
          if (c >= m) break;
#pragma unroll
          for (int q = 0; q < kPanel; ++q)
            if (q < P) cfv[q] = coefs[q * nf + c + P - q - 1];
        }
      }
    }
    front_bar<NT>();
    j += P;
  }
  scale_deferred();
  front_bar<NT>();
  // lower triangle back to the factor storage, except the diagonal blocks of L11 (inverted below)
  for (int k = 0; k < nf; ++k) {
    const T* sk = col(k);
    T* fk = F + (int64_t)k * nf;
    for (int i = k + tid; i < nf; i += NT) {
      if (i < ns && (i >> 5) == (k >> 5)) continue;
      fk[i] = sk[i];
    }
  }
  // inverses of the diagonal blocks: lane j of a warp computes column j of L_blk^-1
  const int nblk = (ns + 31) >> 5;
  for (int bi = warp; bi < nblk; bi += nwarps) {
    const int k0 = bi * 32, w = min(32, ns - k0);
    if (lane < w) {
      const int j = lane;
      T iv[32];
      iv[j] = inv_s[k0 + j];
      F[(k0 + j) + (int64_t)(k0 + j) * nf] = iv[j];
      for (int i = j + 1; i < w; ++i) {
        typename dot_of<T>::type acc(T(0));
        for (int k = j; k < i; ++k) acc.add(col(k0 + k)[k0 + i], iv[k]);
        iv[i] = -acc.value() * inv_s[k0 + i];
        F[(k0 + i) + (int64_t)(k0 + j) * nf] = iv[i];
      }
    }
  }
}

// packed lower triangle, the reciprocal pivots and a panel's column coefficients
template <typename T>
static size_t fused_smem_bytes(int max_nf, int max_ns) {
  return ((size_t)max_nf * (max_nf + 1) / 2 + (size_t)max_ns + (size_t)kPanel * max_nf) * sizeof(T);
}

// CTA size for fronts up to order max_nf: one warp up to 64, then 2, 4, 8 warps
static int fused_threads(int max_nf) { return max_nf <= 64 ? 32 : (max_nf <= 96 ? 64 : (max_nf <= 128 ? 128 : 256)); }

template <typename T, int NT>
static void launch_front_nt(const int32_t* lev, unsigned count, unsigned nz, size_t sm, const CholSymbolic& s,
                            T* const* Wp, int* d_err, cudaStream_t st) {
  allow_dyn_smem(k_chol_front<T, NT>, sm);
  k_chol_front<T, NT><<<dim3(count, 1, nz), NT, sm, st>>>(lev, s.d_fronts, s.d_relmap, Wp, d_err);
  count_launch();
  VH_CUDA_TRY(cudaGetLastError());
}

template <typename T>
static void launch_front(int max_nf, const int32_t* lev, unsigned count, unsigned nz, size_t sm, const CholSymbolic& s,
                         T* const* Wp, int* d_err, cudaStream_t st) {
  switch (fused_threads(max_nf)) {
    case 32: launch_front_nt<T, 32>(lev, count, nz, sm, s, Wp, d_err, st); break;
    case 64: launch_front_nt<T, 64>(lev, count, nz, sm, s, Wp, d_err, st); break;
    case 128: launch_front_nt<T, 128>(lev, count, nz, sm, s, Wp, d_err, st); break;
    default: launch_front_nt<T, 256>(lev, count, nz, sm, s, Wp, d_err, st); break;
  }
}

// the side streams and events of the concurrent level classes (on the current device)
static void ensure_side_streams(const CholSymbolic& s) {
  if (s.ev_fork) return;
  for (int i = 0; i < CholSymbolic::kSideStreams; ++i) {
    VH_CUDA_TRY(cudaStreamCreateWithFlags(&s.side[i], cudaStreamNonBlocking));
    VH_CUDA_TRY(cudaEventCreateWithFlags(&s.ev_join[i], cudaEventDisableTiming));
  }
  VH_CUDA_TRY(cudaEventCreateWithFlags(&s.ev_fork, cudaEventDisableTiming));
}

// the fronts of level hl too large for one CTA: extend-add of the children's update matrices,
// then blocks of kNB pivots (diagonal block, panel, trailing update), all on stream bs
template <typename T>
static void blocked_level(const CholSymbolic& s, size_t hl, unsigned nz, T* const* Wp, int* d_err, cudaStream_t bs) {
  const unsigned nf = (unsigned)s.levels_blocked[hl].size();
  const int32_t* lev = s.d_levels_blocked[hl];
  if (hl > 0) {
    const unsigned cy = (unsigned)std::min(1024, std::max(1, s.blocked_max_nf[hl]));
    for (int which = 0; which < 2; ++which) {
      k_chol_extend_add<T><<<dim3(nf, cy, nz), 128, 0, bs>>>(lev, s.d_fronts, s.d_relmap, Wp, which);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
    }
  }
  const int max_ns = s.blocked_max_ns[hl];
  const int max_nf = s.blocked_max_nf[hl];
  for (int k0 = 0; k0 < max_ns; k0 += kNB) {
    k_chol_diag<T><<<dim3(nf, 1, nz), 256, 0, bs>>>(lev, s.d_fronts, Wp, k0, d_err);
    count_launch();
    const int rows = max_nf - k0;
    if (rows > 0) {
      k_chol_panel<T><<<dim3(nf, (unsigned)ceil_div(rows, 128), nz), 128, 0, bs>>>(lev, s.d_fronts, Wp, k0);
      count_launch();
      const int nt = (int)ceil_div(rows, kTS);
      k_chol_update<T><<<dim3(nf, (unsigned)(nt * (nt + 1) / 2), nz), 256, 0, bs>>>(lev, s.d_fronts, Wp, k0);
      count_launch();
    }
    VH_CUDA_TRY(cudaGetLastError());
  }
}

template <typename T>
void chol_factor(const CholSymbolic& s, int nfac, const double* const* D, T* const* W, cudaStream_t st) {
  if (s.nfronts == 0 || nfac == 0) return;
  VH_REQUIRE(nfac <= 65535, ERR_BAD_ARG, "too many factors in one batch");
  int* d_err = s.d_err;
  if (nfac > s.tab_cap) {   // device: [D pointers | W pointers], kept with the symbolic structure
    cudaFree(s.d_tab);
    s.d_tab = nullptr;
    s.tab_cap = 0;
    VH_CUDA_TRY(cudaMalloc(&s.d_tab, 2 * (size_t)nfac * sizeof(void*)));
    s.tab_cap = nfac;
  }
  void** tab = s.d_tab;
  std::vector<void*> h(2 * (size_t)nfac);
  for (int i = 0; i < nfac; ++i) {
    h[i] = const_cast<double*>(D[i]);
    h[nfac + i] = W[i];
  }
  {
    VH_CUDA_TRY(cudaMemcpyAsync(tab, h.data(), h.size() * sizeof(void*), cudaMemcpyHostToDevice, st));
    const double* const* Dp = reinterpret_cast<const double* const*>(tab);
    T* const* Wp = reinterpret_cast<T* const*>(tab + nfac);
    VH_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    for (int i = 0; i < nfac; ++i) VH_CUDA_TRY(cudaMemsetAsync(W[i], 0, s.w_total * sizeof(T), st));
    const unsigned nz = (unsigned)nfac;
    k_chol_assemble<T><<<dim3(s.nfronts, 1, nz), 256, 0, st>>>(s.d_fronts, s.d_asm, s.d_asm_q, s.d_asm_c, Dp, Wp);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    for (size_t hl = 0; hl < s.levels.size(); ++hl) {
      // the class with the most fronts runs on st; the level's other classes and its blocked fronts
      // on the side streams (forked from st at the level start, joined into st at its end)
      const auto& cls = s.fused_classes[hl];
      const bool has_blocked = !s.levels_blocked[hl].empty();
      int main_c = -1;
      for (int c = 0; c < (int)cls.size(); ++c)
        if (main_c < 0 || cls[c].count > cls[main_c].count) main_c = c;
      const int nside = (int)cls.size() - (main_c >= 0 ? 1 : 0) + (has_blocked ? 1 : 0);
      bool used[CholSymbolic::kSideStreams] = {};
      int next_side = 0;
      auto side_stream = [&]() -> cudaStream_t {
        const int i = next_side++ % CholSymbolic::kSideStreams;
        if (!used[i]) {
          VH_CUDA_TRY(cudaStreamWaitEvent(s.side[i], s.ev_fork, 0));
          used[i] = true;
        }
        return s.side[i];
      };
      if (nside > 0) {
        ensure_side_streams(s);
        VH_CUDA_TRY(cudaEventRecord(s.ev_fork, st));
      }
      for (int c = 0; c < (int)cls.size(); ++c) {
        if (c == main_c) continue;
        const auto& fc = cls[c];
        launch_front<T>(fc.max_nf, s.d_levels_fused[hl] + fc.offset, (unsigned)fc.count, nz,
                        fused_smem_bytes<T>(fc.max_nf, fc.max_ns), s, Wp, d_err, side_stream());
      }
      cudaStream_t bs = has_blocked ? side_stream() : st;
      if (main_c >= 0) {
        const auto& fc = cls[main_c];
        launch_front<T>(fc.max_nf, s.d_levels_fused[hl] + fc.offset, (unsigned)fc.count, nz,
                        fused_smem_bytes<T>(fc.max_nf, fc.max_ns), s, Wp, d_err, st);
      }
      if (has_blocked) blocked_level<T>(s, hl, nz, Wp, d_err, bs);
      for (int i = 0; i < CholSymbolic::kSideStreams; ++i)
        if (used[i]) {
          VH_CUDA_TRY(cudaEventRecord(s.ev_join[i], s.side[i]));
          VH_CUDA_TRY(cudaStreamWaitEvent(st, s.ev_join[i], 0));
        }
    }
    int herr = 0;
    VH_CUDA_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    VH_REQUIRE(herr == 0, ERR_BAD_ARG, "Schur complement is not positive definite (check the port/ground nodes)");
  }
}

// ---- triangular solves.  One warp per (front, RHS), kSolveWarps warps per CTA.  Each front's
// dense triangle is processed in blocks of 32 columns: the 32 x 32 diagonal block is applied as
// its stored inverse (lane i owns row i of the block); the rest is coalesced column-major GEMV /
// dot work whose loads are independent of one another.
constexpr int kSolveWarps = 4;
constexpr int kBlk = 32;
// levels whose largest factor panel (nf x ns entries) fits this many bytes per warp stage the panel
// in shared memory with cp.async at the start of the solve (its loads overlap the gather), so the
// dependent block-by-block reads that follow hit shared memory
constexpr size_t kStagePanelBytes = 24 * 1024;
// the pair-precision forward solve holds kSub entries of a factor row in registers at a time, which
// keeps the unstaged kernel within the register budget of kFsolveCtasPerSm resident CTAs (more
// warps to hide the load latency); the staged kernel's shared memory allows fewer CTAs anyway
constexpr int kSub = 16;
constexpr int kFsolveCtasPerSm = 6;
// the unstaged pair-precision backward solve: shared memory (vector + 32 x 33 block per warp) of the
// leaf level's fronts allows five CTAs per SM, and the registers are held to that
constexpr int kBsolveCtasPerSm = 5;
// the warp-per-front backward solve reads its panels from global memory at every level (staging them
// in shared memory, as the forward solve does, left the staged levels at one CTA per SM)
constexpr bool kStageBackward = false;

__device__ __forceinline__ void cp_async8(void* s, const void* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit_wait() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <typename T>
struct SolveSmem {
  using C = cplx<T>;
  static __host__ __device__ size_t vec_bytes(int max_nf) { return ((size_t)max_nf * sizeof(C) + 15) & ~(size_t)15; }
  static __host__ __device__ size_t panel_bytes(int max_panel) { return ((size_t)max_panel * sizeof(T) + 15) & ~(size_t)15; }
  static __host__ __device__ size_t per_warp(int max_nf, int max_panel = 0) {   // backward: vector, block, y, panel
    return vec_bytes(max_nf) + kBlk * (kBlk + 1) * sizeof(T) + kBlk * sizeof(C) + panel_bytes(max_panel);
  }
  static __host__ __device__ size_t per_warp_fwd(int max_nf, int max_panel = 0) {
    return vec_bytes(max_nf) + kBlk * sizeof(C) + panel_bytes(max_panel);
  }
};

template <typename T, bool STAGE>
__global__ void __launch_bounds__(32 * kSolveWarps, std::is_same<T, double>::value ? 4 : (STAGE ? 5 : kFsolveCtasPerSm))
    k_chol_fsolve(const int32_t* __restrict__ lev, int nlev, int B, const FrontInfo* __restrict__ fr,
                  const int32_t* __restrict__ rows, const int32_t* __restrict__ relmap, T* const* __restrict__ Wp,
                  cplx<T>* __restrict__ x, int64_t ldx, int64_t xoff, cplx<T>* __restrict__ U, int64_t u_total,
                  int max_nf, int max_panel) {
  using C = cplx<T>;
  using Dot = typename dot_of<T>::type;
  constexpr int SUB = std::is_same<T, double>::value ? kBlk : kSub;   // row entries held in registers
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t item = (int64_t)blockIdx.x * kSolveWarps + warp;
  if (item >= (int64_t)nlev * B) return;
  unsigned char* base = smem_raw + warp * SolveSmem<T>::per_warp_fwd(max_nf, STAGE ? max_panel : 0);
  C* t = reinterpret_cast<C*>(base);
  C* yb = reinterpret_cast<C*>(base + SolveSmem<T>::vec_bytes(max_nf));
  T* panel = reinterpret_cast<T*>(yb + kBlk);
  const FrontInfo f = fr[lev[item % nlev]];
  const int b = (int)(item / nlev);
  const T* F = Wp[b] + f.w_off;
  if constexpr (STAGE) {   // the first ns columns (rows 0..nf-1) are all the solve reads
    for (int e = lane; e < f.nf * f.ns; e += 32) cp_async8(panel + e, F + e);
  }
  C* xb = x + b * ldx + xoff;
  C* Ub = U + b * u_total;
  const int32_t* rw = rows + f.rows_off;
  const int nf = f.nf, ns = f.ns;
  // gathers: 4 independent index loads, then 4 independent value loads per lane
  for (int r0 = lane; r0 < nf; r0 += 128) {
    int32_t ix[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) ix[u] = (r0 + 32 * u < ns) ? rw[r0 + 32 * u] : -1;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (r0 + 32 * u < nf) t[r0 + 32 * u] = ix[u] >= 0 ? xb[ix[u]] : czero<C>();
  }
  __syncwarp();
  for (int c = 0; c < 2; ++c) {
    if (f.child[c] < 0) continue;
    const FrontInfo ch = fr[f.child[c]];
    const int32_t* rm = relmap + ch.relmap_off;
    for (int a0 = lane; a0 < ch.nb; a0 += 128) {
      int32_t ix[4];
      C u[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int a = a0 + 32 * q;
        ix[q] = a < ch.nb ? rm[a] : -1;
        u[q] = a < ch.nb ? Ub[ch.u_off + a] : czero<C>();
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (ix[q] >= 0) {
          t[ix[q]].x -= u[q].x;
          t[ix[q]].y -= u[q].y;
        }
    }
    __syncwarp();
  }
  if constexpr (STAGE) {
    cp_async_commit_wait();
    __syncwarp();
    F = panel;
  }
  for (int j0 = 0; j0 < ns; j0 += kBlk) {
    const int w = min(kBlk, ns - j0);
    // the diagonal block holds L_blk^-1: y_blk = L_blk^-1 t_blk, lane i owns row i (its 32 entries
    // are loaded straight into registers: coalesced across lanes for each k)
    {
      yb[lane] = lane < w ? t[j0 + lane] : czero<C>();   // every lane: yb is read for all 32 k
      __syncwarp();
      Dot tx(T(0)), ty(T(0));
#pragma unroll
      for (int h = 0; h < kBlk; h += SUB) {   // SUB entries of the row in registers at a time
        if (h >= w) break;
        T lv[SUB];
#pragma unroll
        for (int k = 0; k < SUB; ++k) {
          const int kk = h + k;
          lv[k] = (kk < w && lane < w && lane >= kk) ? F[(j0 + lane) + (int64_t)(j0 + kk) * nf] : T(0);
        }
#pragma unroll
        for (int k = 0; k < SUB; ++k) {
          if (h + k >= w) break;
          tx.add(lv[k], yb[h + k].x);
          ty.add(lv[k], yb[h + k].y);
        }
      }
      C tv;
      tv.x = tx.value();
      tv.y = ty.value();
      __syncwarp();
      if (lane < w) t[j0 + lane] = tv;
      yb[lane] = tv;   // zero for lanes >= w (their rows are zero); the GEMV below reads all 32
    }
    __syncwarp();
    for (int r = j0 + w + lane; r < nf; r += 32) {
      const T* Lr = F + r + (int64_t)j0 * nf;
      Dot ax(t[r].x), ay(t[r].y);   // t_r - sum_k L(r, k) y_k
#pragma unroll
      for (int h = 0; h < kBlk; h += SUB) {
        if (h >= w) break;   // a partial block stops at w (warp-uniform); zero terms add nothing
        T lv[SUB];
#pragma unroll
        for (int k = 0; k < SUB; ++k) lv[k] = h + k < w ? Lr[(int64_t)(h + k) * nf] : T(0);   // independent loads
#pragma unroll
        for (int k = 0; k < SUB; ++k) {
          if (SUB < kBlk && h + k >= w) break;   // (FP64: one full-width pass, no early exit)
          ax.add(-lv[k], yb[h + k].x);
          ay.add(-lv[k], yb[h + k].y);
        }
      }
      t[r].x = ax.value();
      t[r].y = ay.value();
    }
    __syncwarp();
  }
  for (int j = lane; j < ns; j += 32) xb[rw[j]] = t[j];
  for (int a = lane; a < f.nb; a += 32) {
    const C v = t[ns + a];
    C nv;
    nv.x = -v.x;
    nv.y = -v.y;
    Ub[f.u_off + a] = nv;
  }
}

// Lb[c][r] = L(r0 + r, c0 + c) for r < wr, c < wc of a column-major panel with leading dimension
// nf: lane r loads row r0 + r, one load per column (each coalesced across the lanes), and stores it
// down a column of the padded block, so that lane c can then read column c0 + c without conflicts.
template <typename T>
__device__ __forceinline__ void tile_to_smem(const T* F, int nf, int r0, int c0, int wr, int wc, T (*Lb)[kBlk + 1],
                                             int lane) {
  if (lane < wr) {
    const T* p = F + (r0 + lane) + (int64_t)c0 * nf;
#pragma unroll
    for (int h = 0; h < kBlk; h += 16) {   // 16 independent loads in flight per lane
      if (h >= wc) break;
      T v[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        if (h + c >= wc) break;
        v[c] = p[(int64_t)(h + c) * nf];
      }
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        if (h + c >= wc) break;
        Lb[h + c][lane] = v[c];
      }
    }
  }
}

template <typename T, bool STAGE>
__global__ void __launch_bounds__(32 * kSolveWarps, (STAGE || std::is_same<T, double>::value) ? 1 : kBsolveCtasPerSm)
    k_chol_bsolve(const int32_t* __restrict__ lev, int nlev, int B, const FrontInfo* __restrict__ fr,
                  const int32_t* __restrict__ rows, T* const* __restrict__ Wp, cplx<T>* __restrict__ x, int64_t ldx,
                  int64_t xoff, int max_nf, double2* __restrict__ xd, int64_t ldxd, int max_panel) {
  using C = cplx<T>;
  using Dot = typename dot_of<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t item = (int64_t)blockIdx.x * kSolveWarps + warp;
  if (item >= (int64_t)nlev * B) return;
  unsigned char* base = smem_raw + warp * SolveSmem<T>::per_warp(max_nf, STAGE ? max_panel : 0);
  C* t = reinterpret_cast<C*>(base);
  T(*Lb)[kBlk + 1] = reinterpret_cast<T(*)[kBlk + 1]>(base + SolveSmem<T>::vec_bytes(max_nf));
  T* panel = reinterpret_cast<T*>(base + SolveSmem<T>::vec_bytes(max_nf) + kBlk * (kBlk + 1) * sizeof(T) +
                                  kBlk * sizeof(C));
  const FrontInfo f = fr[lev[item % nlev]];
  const int b = (int)(item / nlev);
  const T* F = Wp[b] + f.w_off;
  if constexpr (STAGE) {
    for (int e = lane; e < f.nf * f.ns; e += 32) cp_async8(panel + e, F + e);
  }
  C* xb = x + b * ldx + xoff;
  const int32_t* rw = rows + f.rows_off;
  const int nf = f.nf, ns = f.ns;
  // own rows: y; boundary rows: final x (4 independent index loads, then value loads, per lane)
  for (int r0 = lane; r0 < nf; r0 += 128) {
    int32_t ix[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) ix[u] = (r0 + 32 * u < nf) ? rw[r0 + 32 * u] : -1;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (ix[u] >= 0) t[r0 + 32 * u] = xb[ix[u]];
  }
  __syncwarp();
  if constexpr (STAGE) {
    cp_async_commit_wait();
    __syncwarp();
    F = panel;
  }
  // z_own -= L21^T x_bnd: lane j accumulates column c0 + j over the boundary rows in order.  Each
  // 32 x 32 tile of L21 is read coalesced (lane = row, one load per column) into the padded block
  // Lb and read back transposed, so no lane walks a column of the column-major panel alone.
  for (int c0 = 0; c0 < ns; c0 += kBlk) {
    const int wc = min(kBlk, ns - c0);
    const C z0 = lane < wc ? t[c0 + lane] : czero<C>();
    Dot sx(z0.x), sy(z0.y);   // z_j - sum_r L(r, j) x_r
    for (int r0 = ns; r0 < nf; r0 += kBlk) {
      const int wr = min(kBlk, nf - r0);
      tile_to_smem<T>(F, nf, r0, c0, wr, wc, Lb, lane);
      __syncwarp();
#pragma unroll 8
      for (int k = 0; k < wr; ++k) {
        const T l = Lb[lane][k];
        const C xr = t[r0 + k];
        sx.add(-l, xr.x);
        sy.add(-l, xr.y);
      }
      __syncwarp();
    }
    if (lane < wc) {
      t[c0 + lane].x = sx.value();
      t[c0 + lane].y = sy.value();
    }
  }
  __syncwarp();
  const int nblk = (ns + kBlk - 1) / kBlk;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int j0 = bi * kBlk;
    const int w = min(kBlk, ns - j0);
    // x_blk = L_blk^-T z_blk with the stored inverse (lower): lane i: x_i = sum_{k >= i} Linv(k, i) z_k
#pragma unroll
    for (int k = 0; k < kBlk; ++k)
      Lb[lane][k] = (k < w && lane < w && lane >= k) ? F[(j0 + lane) + (int64_t)(j0 + k) * nf] : T(0);
    __syncwarp();
    Dot xx(T(0)), xy(T(0));
#pragma unroll 4   // a serial Dot2 chain: unrolling further adds code, not overlap
    for (int k = 0; k < kBlk; ++k) {
      if (k < w) {
        const T l = Lb[k][lane];
        const C zk = t[j0 + k];
        xx.add(l, zk.x);
        xy.add(l, zk.y);
      }
    }
    C xv;
    xv.x = xx.value();
    xv.y = xy.value();
    __syncwarp();
    if (lane < w) t[j0 + lane] = xv;
    __syncwarp();
    // z_j -= sum_{r in block} L(r, j) x_r for the own columns j < j0 (lane per column, the block's
    // rows read as transposed tiles like the boundary rows above)
    for (int c0 = 0; c0 < j0; c0 += kBlk) {
      tile_to_smem<T>(F, nf, j0, c0, w, kBlk, Lb, lane);
      __syncwarp();
      const C zj = t[c0 + lane];
      Dot sx(zj.x), sy(zj.y);
#pragma unroll 8
      for (int k = 0; k < w; ++k) {
        const T l = Lb[lane][k];
        const C xr = t[j0 + k];
        sx.add(-l, xr.x);
        sy.add(-l, xr.y);
      }
      __syncwarp();
      t[c0 + lane].x = sx.value();
      t[c0 + lane].y = sy.value();
    }
    __syncwarp();
  }
  for (int j = lane; j < ns; j += 32) {
    xb[rw[j]] = t[j];
    if (xd) xd[b * ldxd + rw[j]] = to_d(t[j]);   // final value, also in FP64 for the caller
  }
}

// ---- wide triangular solves for the levels near the root, where a few large fronts leave most
// of the GPU idle and one warp per (front, RHS) walks long serial chains: one CTA of kWideWarps
// warps per (front, RHS).  Forward: warp 0 applies the diagonal block, all warps share the rows
// of the block's GEMV.  Backward: the boundary dot products go one warp per column (lanes split
// the rows: coalesced loads, then a shuffle sum), the diagonal block on warp 0 and the block's
// column updates one thread per column.
constexpr int kWideWarps = 8;
constexpr size_t kWarpSolveSmemMax = 160 * 1024;   // warp-per-front CTAs above this go wide
constexpr int kWideMaxFronts = 16;   // levels with at most this many fronts take the wide kernels
constexpr int kWideItemsPerSm = 4;   // ... and levels with at most this many (front, RHS) items per SM

template <typename T>
struct WideSmem {
  using C = cplx<T>;
  static __host__ __device__ size_t vec_bytes(int max_nf) { return ((size_t)max_nf * sizeof(C) + 15) & ~(size_t)15; }
  static __host__ __device__ size_t bytes(int max_nf) {
    return vec_bytes(max_nf) + kBlk * (kBlk + 1) * sizeof(T) + kBlk * sizeof(C);
  }
};

// The wide kernels stage the front's panel (its ns columns, rows 0..nf-1) in shared memory when it
// fits (STAGE): every column is copied with cp.async at the start, overlapping the gathers, so the
// block-by-block chain that follows reads shared memory instead of making two dependent global
// round trips per 32-column block.  The staged panel's leading dimension is odd, so that lanes
// walking columns (the backward updates) hit distinct banks.
constexpr size_t kWideStageMax = 220 * 1024;   // shared memory of a staged wide CTA
constexpr size_t kPipeSmemMax = 224 * 1024;    // ... and of a slab-pipelined one
__host__ __device__ __forceinline__ int staged_ld(int nf) { return nf | 1; }

template <typename T>
__device__ __forceinline__ void stage_panel(T* panel, const T* F, int nf, int ns, int ldp, int warp, int lane) {
  for (int c = warp; c < ns; c += kWideWarps)
    for (int r = lane; r < nf; r += 32) cp_async8(panel + r + (int64_t)c * ldp, F + r + (int64_t)c * nf);
}

template <typename T, bool STAGE>
__global__ void __launch_bounds__(32 * kWideWarps)
    k_chol_fsolve_wide(const int32_t* __restrict__ lev, int nlev, const FrontInfo* __restrict__ fr,
                       const int32_t* __restrict__ rows, const int32_t* __restrict__ relmap, T* const* __restrict__ Wp,
                       cplx<T>* __restrict__ x, int64_t ldx, int64_t xoff, cplx<T>* __restrict__ U, int64_t u_total,
                       int max_nf) {
  using C = cplx<T>;
  using Dot = typename dot_of<T>::type;
  constexpr int NT = 32 * kWideWarps;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* t = reinterpret_cast<C*>(smem_raw);
  C* yb = reinterpret_cast<C*>(smem_raw + WideSmem<T>::vec_bytes(max_nf));
  T* panel = reinterpret_cast<T*>(smem_raw + WideSmem<T>::bytes(max_nf));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const FrontInfo f = fr[lev[blockIdx.x % nlev]];
  const int b = (int)(blockIdx.x / nlev);
  const T* F = Wp[b] + f.w_off;
  C* xb = x + b * ldx + xoff;
  C* Ub = U + b * u_total;
  const int32_t* rw = rows + f.rows_off;
  const int nf = f.nf, ns = f.ns;
  int ld = nf;
  if constexpr (STAGE) stage_panel(panel, F, nf, ns, staged_ld(nf), warp, lane);
  for (int r = tid; r < nf; r += NT) t[r] = r < ns ? xb[rw[r]] : czero<C>();
  __syncthreads();
  for (int c = 0; c < 2; ++c) {
    if (f.child[c] < 0) continue;
    const FrontInfo ch = fr[f.child[c]];
    const int32_t* rm = relmap + ch.relmap_off;
    for (int a = tid; a < ch.nb; a += NT) {   // distinct targets within one child
      const C u = Ub[ch.u_off + a];
      C& tv = t[rm[a]];
      tv.x -= u.x;
      tv.y -= u.y;
    }
    __syncthreads();
  }
  if constexpr (STAGE) {
    cp_async_commit_wait();
    __syncthreads();
    F = panel;
    ld = staged_ld(nf);
  }
  for (int j0 = 0; j0 < ns; j0 += kBlk) {
    const int w = min(kBlk, ns - j0);
    if (warp == 0) {   // y_blk = L_blk^-1 t_blk (stored inverse), lane i owns row i
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        lv[k] = (k < w && lane < w && lane >= k) ? F[(j0 + lane) + (int64_t)(j0 + k) * ld] : T(0);
      yb[lane] = lane < w ? t[j0 + lane] : czero<C>();
      __syncwarp();
      Dot tx(T(0)), ty(T(0));
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        if (k < w) {
          tx.add(lv[k], yb[k].x);
          ty.add(lv[k], yb[k].y);
        }
      C tv;
      tv.x = tx.value();
      tv.y = ty.value();
      __syncwarp();
      if (lane < w) t[j0 + lane] = tv;
      yb[lane] = tv;
    }
    __syncthreads();
    // the block's update of the pivot rows below it (the boundary rows follow in one pass)
    for (int r = j0 + w + tid; r < ns; r += NT) {
      const T* Lr = F + r + (int64_t)j0 * ld;
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k) lv[k] = k < w ? Lr[(int64_t)k * ld] : T(0);
      Dot ax(t[r].x), ay(t[r].y);
#pragma unroll
      for (int k = 0; k < kBlk; ++k) {
        ax.add(-lv[k], yb[k].x);
        ay.add(-lv[k], yb[k].y);
      }
      t[r].x = ax.value();
      t[r].y = ay.value();
    }
    __syncthreads();
  }
  // the boundary rows: t_r -= sum_{j < ns} L(r, j) y_j in one pass over the front's off-diagonal part
  // (each thread a row, the columns in groups of kBlk loads in flight), instead of one slice per
  // block step: the steps above then walk only the pivot rows
  for (int r = ns + tid; r < nf; r += NT) {
    Dot ax(t[r].x), ay(t[r].y);
    for (int j0 = 0; j0 < ns; j0 += kBlk) {
      const int w = min(kBlk, ns - j0);
      const T* Lr = F + r + (int64_t)j0 * ld;
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k) lv[k] = k < w ? Lr[(int64_t)k * ld] : T(0);
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        if (k < w) {
          const C y = t[j0 + k];
          ax.add(-lv[k], y.x);
          ay.add(-lv[k], y.y);
        }
    }
    t[r].x = ax.value();
    t[r].y = ay.value();
  }
  __syncthreads();
  for (int j = tid; j < ns; j += NT) xb[rw[j]] = t[j];
  for (int a = tid; a < f.nb; a += NT) {
    const C v = t[ns + a];
    C nv;
    nv.x = -v.x;
    nv.y = -v.y;
    Ub[f.u_off + a] = nv;
  }
}

// The wide forward solve for fronts too large to stage whole: the pivot-block steps read 32-column
// slabs of the panel (columns j0 .. j0 + 31, rows j0 .. ns - 1) from shared memory, and the next slab
// is copied with cp.async while the current step computes (two slabs of `sl` rows), so that no step
// waits on global memory; the boundary rows then take one streaming pass over the off-diagonal part.
template <typename T>
struct PipeSmem {
  static __host__ __device__ size_t bytes(int max_nf, int sl) {
    return WideSmem<T>::vec_bytes(max_nf) + ((kBlk * sizeof(cplx<T>) + 15) & ~(size_t)15) +
           2 * (size_t)kBlk * sl * sizeof(T);
  }
};

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <typename T>
__global__ void __launch_bounds__(32 * kWideWarps)
    k_chol_fsolve_wide_pipe(const int32_t* __restrict__ lev, int nlev, const FrontInfo* __restrict__ fr,
                            const int32_t* __restrict__ rows, const int32_t* __restrict__ relmap,
                            T* const* __restrict__ Wp, cplx<T>* __restrict__ x, int64_t ldx, int64_t xoff,
                            cplx<T>* __restrict__ U, int64_t u_total, int max_nf, int sl) {
  using C = cplx<T>;
  using Dot = typename dot_of<T>::type;
  constexpr int NT = 32 * kWideWarps;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* t = reinterpret_cast<C*>(smem_raw);
  C* yb = reinterpret_cast<C*>(smem_raw + WideSmem<T>::vec_bytes(max_nf));
  T* slab0 = reinterpret_cast<T*>(smem_raw + WideSmem<T>::vec_bytes(max_nf) +
                                  ((kBlk * sizeof(C) + 15) & ~(size_t)15));
  T* slabs[2] = {slab0, slab0 + (size_t)kBlk * sl};
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const FrontInfo f = fr[lev[blockIdx.x % nlev]];
  const int b = (int)(blockIdx.x / nlev);
  const T* F = Wp[b] + f.w_off;
  C* xb = x + b * ldx + xoff;
  C* Ub = U + b * u_total;
  const int32_t* rw = rows + f.rows_off;
  const int nf = f.nf, ns = f.ns;
  auto stage = [&](int j0, T* dst) {   // slab of step j0: element (i, k) = L(j0 + i, j0 + k) at dst[k sl + i]
    const int w = min(kBlk, ns - j0), h = ns - j0;
    for (int q = tid; q < w * h; q += NT) {
      const int k = q / h, i = q - k * h;
      cp_async8(dst + k * sl + i, F + (j0 + i) + (int64_t)(j0 + k) * nf);
    }
    cp_async_commit();
  };
  stage(0, slabs[0]);
  for (int r = tid; r < nf; r += NT) t[r] = r < ns ? xb[rw[r]] : czero<C>();
  __syncthreads();
  for (int c = 0; c < 2; ++c) {
    if (f.child[c] < 0) continue;
    const FrontInfo ch = fr[f.child[c]];
    const int32_t* rm = relmap + ch.relmap_off;
    for (int a = tid; a < ch.nb; a += NT) {   // distinct targets within one child
      const C u = Ub[ch.u_off + a];
      C& tv = t[rm[a]];
      tv.x -= u.x;
      tv.y -= u.y;
    }
    __syncthreads();
  }
  int buf = 0;
  for (int j0 = 0; j0 < ns; j0 += kBlk, buf ^= 1) {
    const int w = min(kBlk, ns - j0);
    cp_async_wait0();
    __syncthreads();   // slab j0 in shared memory; every thread is done with the previous step
    if (j0 + kBlk < ns) stage(j0 + kBlk, slabs[buf ^ 1]);
    const T* S = slabs[buf];
    if (warp == 0) {   // y_blk = L_blk^-1 t_blk (stored inverse), lane i owns row i
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k) lv[k] = (k < w && lane < w && lane >= k) ? S[k * sl + lane] : T(0);
      yb[lane] = lane < w ? t[j0 + lane] : czero<C>();
      __syncwarp();
      Dot tx(T(0)), ty(T(0));
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        if (k < w) {
          tx.add(lv[k], yb[k].x);
          ty.add(lv[k], yb[k].y);
        }
      C tv;
      tv.x = tx.value();
      tv.y = ty.value();
      __syncwarp();
      if (lane < w) t[j0 + lane] = tv;
      yb[lane] = tv;
    }
    __syncthreads();
    for (int r = j0 + w + tid; r < ns; r += NT) {
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k) lv[k] = k < w ? S[k * sl + (r - j0)] : T(0);
      Dot ax(t[r].x), ay(t[r].y);
#pragma unroll
      for (int k = 0; k < kBlk; ++k) {
        ax.add(-lv[k], yb[k].x);
        ay.add(-lv[k], yb[k].y);
      }
      t[r].x = ax.value();
      t[r].y = ay.value();
    }
  }
  __syncthreads();
  for (int r = ns + tid; r < nf; r += NT) {   // the boundary rows in one pass (as k_chol_fsolve_wide)
    Dot ax(t[r].x), ay(t[r].y);
    for (int j0 = 0; j0 < ns; j0 += kBlk) {
      const int w = min(kBlk, ns - j0);
      const T* Lr = F + r + (int64_t)j0 * nf;
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k) lv[k] = k < w ? Lr[(int64_t)k * nf] : T(0);
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        if (k < w) {
          const C y = t[j0 + k];
          ax.add(-lv[k], y.x);
          ay.add(-lv[k], y.y);
        }
    }
    t[r].x = ax.value();
    t[r].y = ay.value();
  }
  __syncthreads();
  for (int j = tid; j < ns; j += NT) xb[rw[j]] = t[j];
  for (int a = tid; a < f.nb; a += NT) {
    const C v = t[ns + a];
    C nv;
    nv.x = -v.x;
    nv.y = -v.y;
    Ub[f.u_off + a] = nv;
  }
}

template <typename T, bool STAGE>
__global__ void __launch_bounds__(32 * kWideWarps)
    k_chol_bsolve_wide(const int32_t* __restrict__ lev, int nlev, const FrontInfo* __restrict__ fr,
                       const int32_t* __restrict__ rows, T* const* __restrict__ Wp, cplx<T>* __restrict__ x,
                       int64_t ldx, int64_t xoff, int max_nf, double2* __restrict__ xd, int64_t ldxd) {
  using C = cplx<T>;
  using Dot = typename dot_of<T>::type;
  constexpr int NT = 32 * kWideWarps;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* t = reinterpret_cast<C*>(smem_raw);
  T(*Lb)[kBlk + 1] = reinterpret_cast<T(*)[kBlk + 1]>(smem_raw + WideSmem<T>::vec_bytes(max_nf));
  T* panel = reinterpret_cast<T*>(smem_raw + WideSmem<T>::bytes(max_nf));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const FrontInfo f = fr[lev[blockIdx.x % nlev]];
  const int b = (int)(blockIdx.x / nlev);
  const T* F = Wp[b] + f.w_off;
  C* xb = x + b * ldx + xoff;
  const int32_t* rw = rows + f.rows_off;
  const int nf = f.nf, ns = f.ns;
  int ld = nf;
  if constexpr (STAGE) stage_panel(panel, F, nf, ns, staged_ld(nf), warp, lane);
  for (int r = tid; r < nf; r += NT) t[r] = xb[rw[r]];
  if constexpr (STAGE) {
    cp_async_commit_wait();
    F = panel;
    ld = staged_ld(nf);
  }
  __syncthreads();
  // z_j -= sum_{r >= ns} L(r, j) x_r: warp per column, lanes over the rows, then a shuffle sum
  for (int j = warp; j < ns; j += kWideWarps) {
    const T* col = F + (int64_t)j * ld;
    Dot sx(T(0)), sy(T(0));
    for (int r = ns + lane; r < nf; r += 32) {
      const T l = col[r];
      sx.add(l, t[r].x);
      sy.add(l, t[r].y);
    }
    sx.warp_sum();
    sy.warp_sum();
    if (lane == 0) {
      Dot zx(t[j].x), zy(t[j].y);
      zx.add(T(-1), sx.value());
      zy.add(T(-1), sy.value());
      t[j].x = zx.value();
      t[j].y = zy.value();
    }
  }
  __syncthreads();
  const int nblk = (ns + kBlk - 1) / kBlk;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int j0 = bi * kBlk;
    const int w = min(kBlk, ns - j0);
    if (warp == 0) {   // x_blk = L_blk^-T z_blk: lane i: x_i = sum_{k >= i} Linv(k, i) z_k
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        Lb[lane][k] = (k < w && lane < w && lane >= k) ? F[(j0 + lane) + (int64_t)(j0 + k) * ld] : T(0);
      __syncwarp();
      Dot xx(T(0)), xy(T(0));
#pragma unroll 4   // one serial Dot2 chain, as in k_chol_bsolve
      for (int k = 0; k < kBlk; ++k)
        if (k < w) {
          const T l = Lb[k][lane];
          const C zk = t[j0 + k];
          xx.add(l, zk.x);
          xy.add(l, zk.y);
        }
      C xv;
      xv.x = xx.value();
      xv.y = xy.value();
      __syncwarp();
      if (lane < w) t[j0 + lane] = xv;
    }
    __syncthreads();
    for (int j = tid; j < j0; j += NT) {   // z_j -= sum_{k in block} L(j0 + k, j) x_{j0 + k}
      const T* col = F + (int64_t)j * ld + j0;
      T lv[kBlk];
#pragma unroll
      for (int k = 0; k < kBlk; ++k) lv[k] = k < w ? col[k] : T(0);
      Dot sx(t[j].x), sy(t[j].y);
#pragma unroll
      for (int k = 0; k < kBlk; ++k)
        if (k < w) {
          sx.add(-lv[k], t[j0 + k].x);
          sy.add(-lv[k], t[j0 + k].y);
        }
      t[j].x = sx.value();
      t[j].y = sy.value();
    }
    __syncthreads();
  }
  for (int j = tid; j < ns; j += NT) {
    xb[rw[j]] = t[j];
    if (xd) xd[b * ldxd + rw[j]] = to_d(t[j]);
  }
}

template <typename T>
void chol_solve(const CholSymbolic& s, int B, T* const* Wp, cplx<T>* x, int64_t ldx, int64_t xoff, cplx<T>* U,
                cudaStream_t st, double2* xd, int64_t ldxd) {
  if (s.nfronts == 0 || B == 0) return;
  const int stage_max = (int)(kStagePanelBytes / sizeof(T));   // panel entries a warp may stage
  auto panel = [&](size_t h) { return s.level_max_nf[h] * s.level_max_ns[h]; };   // bounds every front's nf * ns
  auto stage = [&](size_t h) { return panel(h) <= stage_max; };
  auto warp_smem = [&](size_t h, bool fwd) {
    const int mp = stage(h) ? panel(h) : 0;
    return kSolveWarps * (fwd ? SolveSmem<T>::per_warp_fwd(s.level_max_nf[h], mp)
                              : SolveSmem<T>::per_warp(s.level_max_nf[h], mp));
  };
  // a level of few fronts, or of fronts whose per-warp vectors do not fit four to a CTA, takes the
  // wide kernels (one CTA per front and RHS)
  // ... or a level whose (front, RHS) items number at most kWideItemsPerSm per SM: one warp per item
  // would leave each SM a few warps streaming long panels (measured on the ring and two-bar sweeps:
  // 400-800 items at 152 SMs cut the apply by 7-10 %, 3200 items lost again)
  static const int64_t wide_items = [] {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    return (int64_t)kWideItemsPerSm * sms;
  }();
  auto wide = [&](size_t h) {
    return (int)s.levels[h].size() <= kWideMaxFronts || warp_smem(h, false) > kWarpSolveSmemMax ||
           (int64_t)s.levels[h].size() * B <= wide_items;
  };
  // a wide level stages its panels when the largest (max ns columns of odd leading dimension) fits
  auto wide_smem = [&](size_t h, bool staged) {
    const size_t base = WideSmem<T>::bytes(s.level_max_nf[h]);
    return staged ? base + (size_t)s.level_max_ns[h] * staged_ld(s.level_max_nf[h]) * sizeof(T) : base;
  };
  auto wide_stage = [&](size_t h) { return wide_smem(h, true) <= kWideStageMax; };
  // a wide level too large to stage whole pipelines two 32-column slabs of its panels when they fit
  auto pipe_smem = [&](size_t h) { return PipeSmem<T>::bytes(s.level_max_nf[h], s.level_max_ns[h]); };
  auto pipe_ok = [&](size_t h) { return pipe_smem(h) <= kPipeSmemMax; };
  size_t sm_f[2] = {0, 0}, sm_b[2] = {0, 0}, sm_w[2] = {0, 0}, sm_p = 0;
  for (size_t h = 0; h < s.levels.size(); ++h) {
    if (wide(h)) {
      const bool ws = wide_stage(h);
      sm_w[ws] = std::max(sm_w[ws], wide_smem(h, ws));
      if (!ws && pipe_ok(h)) sm_p = std::max(sm_p, pipe_smem(h));
    } else {
      sm_f[stage(h)] = std::max(sm_f[stage(h)], warp_smem(h, true));
      const bool sb = kStageBackward && stage(h);
      sm_b[sb] = std::max(sm_b[sb], kSolveWarps * SolveSmem<T>::per_warp(s.level_max_nf[h], sb ? panel(h) : 0));
    }
  }
  VH_REQUIRE(sm_w[0] <= kWideStageMax, ERR_UNSUPPORTED, "front too large for the shared-memory solve");
  if (sm_f[0]) allow_dyn_smem(k_chol_fsolve<T, false>, sm_f[0]);
  if (sm_f[1]) allow_dyn_smem(k_chol_fsolve<T, true>, sm_f[1]);
  if (sm_b[0]) allow_dyn_smem(k_chol_bsolve<T, false>, sm_b[0]);
  if (sm_b[1]) allow_dyn_smem(k_chol_bsolve<T, true>, sm_b[1]);
  if (sm_w[0]) {
    allow_dyn_smem(k_chol_fsolve_wide<T, false>, sm_w[0]);
    allow_dyn_smem(k_chol_bsolve_wide<T, false>, sm_w[0]);
  }
  if (sm_w[1]) {
    allow_dyn_smem(k_chol_fsolve_wide<T, true>, sm_w[1]);
    allow_dyn_smem(k_chol_bsolve_wide<T, true>, sm_w[1]);
  }
  if (sm_p) allow_dyn_smem(k_chol_fsolve_wide_pipe<T>, sm_p);
  for (size_t h = 0; h < s.levels.size(); ++h) {
    const int nlev = (int)s.levels[h].size();
    const int mnf = s.level_max_nf[h];
    if (wide(h)) {
      const unsigned g = (unsigned)(nlev * B);
      if (wide_stage(h))
        k_chol_fsolve_wide<T, true><<<g, 32 * kWideWarps, wide_smem(h, true), st>>>(
            s.d_levels[h], nlev, s.d_fronts, s.d_rows, s.d_relmap, Wp, x, ldx, xoff, U, s.u_total, mnf);
      else if (pipe_ok(h))
        k_chol_fsolve_wide_pipe<T><<<g, 32 * kWideWarps, pipe_smem(h), st>>>(
            s.d_levels[h], nlev, s.d_fronts, s.d_rows, s.d_relmap, Wp, x, ldx, xoff, U, s.u_total, mnf,
            s.level_max_ns[h]);
      else
        k_chol_fsolve_wide<T, false><<<g, 32 * kWideWarps, wide_smem(h, false), st>>>(
            s.d_levels[h], nlev, s.d_fronts, s.d_rows, s.d_relmap, Wp, x, ldx, xoff, U, s.u_total, mnf);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      continue;
    }
    const int mp = panel(h);
    const bool stg = stage(h);
    const size_t smh = kSolveWarps * SolveSmem<T>::per_warp_fwd(mnf, stg ? mp : 0);
    const unsigned grid = (unsigned)ceil_div((int64_t)nlev * B, kSolveWarps);
    if (stg)
      k_chol_fsolve<T, true><<<grid, 32 * kSolveWarps, smh, st>>>(s.d_levels[h], nlev, B, s.d_fronts, s.d_rows,
                                                                  s.d_relmap, Wp, x, ldx, xoff, U, s.u_total, mnf, mp);
    else
      k_chol_fsolve<T, false><<<grid, 32 * kSolveWarps, smh, st>>>(s.d_levels[h], nlev, B, s.d_fronts, s.d_rows,
                                                                   s.d_relmap, Wp, x, ldx, xoff, U, s.u_total, mnf, 0);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
  for (size_t hh = s.levels.size(); hh-- > 0;) {
    const int nlev = (int)s.levels[hh].size();
    const int mnf = s.level_max_nf[hh];
    if (wide(hh)) {
      const unsigned g = (unsigned)(nlev * B);
      if (wide_stage(hh))
        k_chol_bsolve_wide<T, true><<<g, 32 * kWideWarps, wide_smem(hh, true), st>>>(
            s.d_levels[hh], nlev, s.d_fronts, s.d_rows, Wp, x, ldx, xoff, mnf, xd, ldxd);

      else
        k_chol_bsolve_wide<T, false><<<g, 32 * kWideWarps, wide_smem(hh, false), st>>>(
            s.d_levels[hh], nlev, s.d_fronts, s.d_rows, Wp, x, ldx, xoff, mnf, xd, ldxd);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      continue;
    }
    const int mp = panel(hh);
    const bool stg = kStageBackward && stage(hh);
    const size_t smh = kSolveWarps * SolveSmem<T>::per_warp(mnf, stg ? mp : 0);
    const unsigned grid = (unsigned)ceil_div((int64_t)nlev * B, kSolveWarps);
    if (stg)
      k_chol_bsolve<T, true><<<grid, 32 * kSolveWarps, smh, st>>>(s.d_levels[hh], nlev, B, s.d_fronts, s.d_rows, Wp,
                                                                  x, ldx, xoff, mnf, xd, ldxd, mp);
    else
      k_chol_bsolve<T, false><<<grid, 32 * kSolveWarps, smh, st>>>(s.d_levels[hh], nlev, B, s.d_fronts, s.d_rows, Wp,
                                                                   x, ldx, xoff, mnf, xd, ldxd, 0);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
  }
}

template void chol_factor<double>(const CholSymbolic&, int, const double* const*, double* const*, cudaStream_t);
template void chol_solve<double>(const CholSymbolic&, int, double* const*, double2*, int64_t, int64_t, double2*,
                                 cudaStream_t, double2*, int64_t);
template void chol_factor<dfloat>(const CholSymbolic&, int, const double* const*, dfloat* const*, cudaStream_t);
template void chol_solve<dfloat>(const CholSymbolic&, int, dfloat* const*, dcomplex*, int64_t, int64_t, dcomplex*,
                                 cudaStream_t, double2*, int64_t);

}  // namespace vh
