// Inputs of the solve path built natively: panel numbering and the incidence matrix Ae (host,
// lse_generate_panelIDs.m / lse_compute_Ae_matrix.m) and the circulant Green tensor (device,
// lse_generate_circulant_tensor.m with lse_enhanced_near = 3, lse_exploit_symmetry = 1).
//
// Tensor quadrature.  volume_volume.m integrates over a 6-D tensor Gauss-Legendre rule; the
// kernel depends on (X - X', Y - Y', Z - Z') only and the test/basis weights are products of
// one-dimensional factors (1, x, x' x).  Grouping the node pairs of each dimension by their
// difference d = x_i - x_j gives one-dimensional tables
//   w0(d) = sum w_i w_j,   w1(d) = sum w_i w_j (h x_i),   w2(d) = sum w_i w_j (h x_j)(h x_i)
// and the 6-D sum becomes a 3-D sum over difference triples: for the 3-point rule 5^3 = 125
// kernel evaluations per offset instead of 3^6 = 729 (same sum, different rounding order).
#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "../../include/voxhenry_gpu.h"
#include "vh_internal.cuh"

namespace vh {

// src_lin_vie/K_near_interactions_1mm.txt: near interactions of a 1 mm voxel at offsets
// (1,1,1),(1,2,1),(1,2,2),(2,1,1),(2,2,1),(2,2,2): pulse-pulse, linear(x)-pulse,
// linear(x)-linear(x'), each (re, im).  Data of the reference, reproduced verbatim.
static const double kNear1mm[6][3][2] = {
    {{1.497896808995041e-016, -5.003461427972696e-027}, {-1.884273158210909e-037, -2.012211605895784e-048}, {2.910077873947119e-024, -3.626541131608855e-051}},
    {{7.805636278778824e-017, -5.003461427972697e-027}, {1.206473223753176e-035, -4.160008679876429e-049}, {6.11217610670709e-025, -2.004923164762494e-052}},
    {{5.638025079837469e-017, -5.003461427972694e-027}, {2.412452305035321e-035, 2.98904327368899e-049}, {2.297463434675418e-025, -5.006665539022287e-052}},
    {{7.805636278778813e-017, -5.003461427972696e-027}, {-5.757414693177654e-021, -7.50496380728818e-048}, {-7.440943011730615e-025, -1.219881017509337e-051}},
    {{5.638025079837419e-017, -5.003461427972694e-027}, {-2.390823543614732e-021, -3.06145823959795e-048}, {-1.275734678285788e-025, 1.681050961223937e-051}},
    {{4.605920193990263e-017, -5.003461427972694e-027}, {-1.321546896796384e-021, 2.534523806813602e-049}, {-1.402863426594222e-026, -1.963545763613549e-051}},
};

// gperiodic_coeff_nop_linJVIE.m: component signs when mirrored across x (L), y (M), z (N).
// Component k is odd in x for k = 2 (G2D,x), in y for k = 3 (G2D,y), in z for k = 5 (G3D,z).
__host__ __device__ inline double mirror_sign(int k, bool fx, bool fy, bool fz) {
  double s = 1.0;
  if (fx && k == 1) s = -s;
  if (fy && k == 2) s = -s;
  if (fz && k == 4) s = -s;
  return s;
}

constexpr double kKoGrfn = 1e-30;   // lse_generate_circulant_tensor.m:21-23

struct DiffTable {
  int n = 0;
  double d[32], w0[32], w1[32], w2[32];
};

// Gauss-Legendre nodes / weights on [-1, 1] (Newton iteration on P_n; Golub-Welsch not needed)
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < (n + 1) / 2; ++i) {
    long double z = cosl(pi * (i + 0.75L) / (n + 0.5L));
    long double dp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const long double pn = (n == 1) ? z : p1, pnm1 = (n == 1) ? 1 : p0;
      dp = n * (z * pn - pnm1) / (z * z - 1);
      const long double dz = pn / dp;
      z -= dz;
      if (fabsl(dz) < 1e-30L) break;
    }
    long double p0 = 1, p1 = z;
    for (int k = 2; k <= n; ++k) {
      const long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1);
    const long double wi = 2 / ((1 - z * z) * dp * dp);
    x[i] = (double)-z;
    x[n - 1 - i] = (double)z;
    w[i] = w[n - 1 - i] = (double)wi;
  }
  if (n % 2) x[n / 2] = 0.0;
}

static DiffTable diff_table(int n, double h) {
  std::vector<double> x, w;
  gauss_legendre(n, x, w);
  std::map<double, int> idx;
  DiffTable t;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double d = x[i] - x[j];
      auto it = idx.find(d);
      int k;
      if (it == idx.end()) {
        k = t.n++;
        idx[d] = k;
        t.d[k] = d;
        t.w0[k] = t.w1[k] = t.w2[k] = 0.0;
      } else {
        k = it->second;
      }
      const double ww = w[i] * w[j];
      t.w0[k] += ww;
      t.w1[k] += ww * (h * x[i]);
      t.w2[k] += ww * ((h * x[j]) * (h * x[i]));
    }
  return t;
}

// One thread per offset (mx, my, mz): the 7 integrals of volume_volume.m:100-115 (unnormalised).
// out: column-major (L, M, N, 7) complex; only offsets with mx < Lc, my < Mc, mz < Nc when `box`.
__global__ void k_volume_volume(DiffTable t, double dx, int L, int M, int N, int Lc, int Mc, int Nc,
                                double2* __restrict__ G) {
  const int64_t cnt = (int64_t)Lc * Mc * Nc;
  const double h = dx / 2;
  const double J = h * h * h * h * h * h;
  const double c4pi = 1.0 / 4.0 / 3.14159265358979323846;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < cnt; o += (int64_t)gridDim.x * blockDim.x) {
    const int mx = o % Lc, my = (o / Lc) % Mc, mz = o / ((int64_t)Lc * Mc);
    const double rx = mx * dx, ry = my * dx, rz = mz * dx;
    double k1r = 0, k1i = 0, k3r = 0, k3i = 0, k5r = 0, k5i = 0, k7r = 0, k7i = 0, k8r = 0, k8i = 0, k9r = 0, k9i = 0,
           k10r = 0, k10i = 0;
    for (int c = 0; c < t.n; ++c) {
      const double ez = rz + h * t.d[c];
      for (int b = 0; b < t.n; ++b) {
        const double ey = ry + h * t.d[b];
        const double wyz00 = t.w0[b] * t.w0[c];
        const double wyz10 = t.w1[b] * t.w0[c], wyz01 = t.w0[b] * t.w1[c];
        const double wyz20 = t.w2[b] * t.w0[c], wyz02 = t.w0[b] * t.w2[c];
        for (int a = 0; a < t.n; ++a) {
          const double ex = rx + h * t.d[a];
          const double R = sqrt(ex * ex + ey * ey + ez * ez);
          double s, co;
          sincos(kKoGrfn * R, &s, &co);
          const double kr = c4pi * co / R, ki = -c4pi * s / R;   // 1/4/pi exp(-j k0 R) / R
          const double w0 = t.w0[a] * wyz00;
          k1r += w0 * kr;  k1i += w0 * ki;
          const double w3 = t.w1[a] * wyz00;
          k3r += w3 * kr;  k3i += w3 * ki;
          const double w5 = t.w0[a] * wyz10;
          k5r += w5 * kr;  k5i += w5 * ki;
          const double w7 = t.w0[a] * wyz01;
          k7r += w7 * kr;  k7i += w7 * ki;
          const double w8 = t.w2[a] * wyz00;
          k8r += w8 * kr;  k8i += w8 * ki;
          const double w9 = t.w0[a] * wyz20;
          k9r += w9 * kr;  k9i += w9 * ki;
          const double w10 = t.w0[a] * wyz02;
          k10r += w10 * kr; k10i += w10 * ki;
        }
      }
    }
    const int64_t P = (int64_t)L * M * N;
    const int64_t li = mx + (int64_t)L * (my + (int64_t)M * mz);
    G[li + 0 * P] = make_double2(k1r * J, k1i * J);
    G[li + 1 * P] = make_double2(-k3r * J, -k3i * J);
    G[li + 2 * P] = make_double2(k5r * J, k5i * J);
    G[li + 3 * P] = make_double2((k8r + k9r) * J, (k8i + k9i) * J);
    G[li + 4 * P] = make_double2(2 * k7r * J, 2 * k7i * J);
    G[li + 5 * P] = make_double2((k8r - k9r) * J, (k8i - k9i) * J);
    G[li + 6 * P] = make_double2((k8r + k9r + 4 * k10r) * J, (k8i + k9i + 4 * k10i) * J);
  }
}

// volume_volume_sym.m (dir = 1): pulse-pulse, lin(x)-pulse, lin(x)-lin(x') at listed offsets.
// One CTA per offset; block reduction over the difference triples.
__global__ void k_volume_volume_sym(DiffTable t, double dx, const int* __restrict__ offs, double2* __restrict__ K) {
  const int o = blockIdx.x;
  const double h = dx / 2;
  const double J = h * h * h * h * h * h;
  const double c4pi = 1.0 / 4.0 / 3.14159265358979323846;
  const double rx = offs[3 * o] * dx, ry = offs[3 * o + 1] * dx, rz = offs[3 * o + 2] * dx;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const int tot = t.n * t.n * t.n;
  for (int q = threadIdx.x; q < tot; q += blockDim.x) {
    const int a = q % t.n, b = (q / t.n) % t.n, c = q / (t.n * t.n);
    const double ex = rx + h * t.d[a], ey = ry + h * t.d[b], ez = rz + h * t.d[c];
    const double R = sqrt(ex * ex + ey * ey + ez * ez);
    double s, co;
    sincos(kKoGrfn * R, &s, &co);
    const double kr = c4pi * co / R, ki = -c4pi * s / R;
    const double wyz = t.w0[b] * t.w0[c];
    const double w0 = t.w0[a] * wyz, w1 = t.w1[a] * wyz, w2 = t.w2[a] * wyz;
    acc[0] += w0 * kr; acc[1] += w0 * ki;
    acc[2] += w1 * kr; acc[3] += w1 * ki;
    acc[4] += w2 * kr; acc[5] += w2 * ki;
  }
  __shared__ double red[6][256];
  for (int i = 0; i < 6; ++i) red[i][threadIdx.x] = acc[i];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int i = 0; i < 6; ++i) red[i][threadIdx.x] += red[i][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int i = 0; i < 3; ++i) K[3 * o + i] = make_double2(red[2 * i][0] * J, red[2 * i + 1][0] * J);
}

// lse_generate_circulant_tensor.m:761-768 normalisation, in place on (L, M, N, 7)
__global__ void k_normalise(double2* __restrict__ G, int64_t P, double dx) {
  const double d4 = dx * dx * dx * dx;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 7 * P; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / P);
    double s = 1.0 / d4;
    double2 v = G[i];
    v.x = v.x / d4;
    v.y = v.y / d4;
    if (k == 1 || k == 2 || k == 4) s = 1.0 / dx;
    else if (k >= 3) s = 1.0 / (dx * dx);
    if (k != 0) {
      v.x *= s;
      v.y *= s;
    }
    G[i] = v;
  }
}

// circulant embedding (lse_generate_circulant_tensor.m:799-816) into column-major (2L, 2M, 2N, 7)
__global__ void k_embed(const double2* __restrict__ G, int L, int M, int N, double2* __restrict__ Gp) {
  const int X = 2 * L, Y = 2 * M, Z = 2 * N;
  const int64_t P = (int64_t)X * Y * Z, PG = (int64_t)L * M * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 7 * P; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / P);
    const int64_t r = i % P;
    const int x = r % X, y = (r / X) % Y, z = r / ((int64_t)X * Y);
    double2 v = make_double2(0.0, 0.0);
    if (x != L && y != M && z != N) {
      const bool fx = x > L, fy = y > M, fz = z > N;
      const int sx = fx ? X - x : x, sy = fy ? Y - y : y, sz = fz ? Z - z : z;
      const double sg = mirror_sign(k, fx, fy, fz);
      const double2 g = G[sx + (int64_t)L * (sy + (int64_t)M * sz) + k * PG];
      v = make_double2(sg * g.x, sg * g.y);
    }
    Gp[i] = v;
  }
}

// ---------------------------------------------------------------------------- host helpers
static void scatter_sym(std::vector<double2>& G5, int n5x, int n5y, int n5z, const std::vector<int>& offs,
                        const std::vector<double2>& K) {
  // G5: column-major (n5x, n5y, n5z, 7) block of G; symmetric fill of lse_generate_circulant_tensor.m:184-305
  auto at = [&](int a, int b, int c, int k) -> double2& { return G5[a + n5x * (b + n5y * (c + (size_t)n5z * k))]; };
  auto add = [](double2& d, double2 v, double s) { d.x += s * v.x; d.y += s * v.y; };
  auto set = [](double2& d, double2 v, double s) { d = make_double2(s * v.x, s * v.y); };
  for (size_t e = 0; e < offs.size() / 3; ++e) {
    const int a = offs[3 * e], b = offs[3 * e + 1], c = offs[3 * e + 2];   // 0-based (mx, my, mz)
    const double2 k1 = K[3 * e], k2 = K[3 * e + 1], k3 = K[3 * e + 2];
    set(at(a, b, c, 0), k1, 1);
    set(at(a, b, c, 1), k2, -1);
    add(at(a, b, c, 3), k3, 1);
    add(at(a, b, c, 5), k3, 1);
    add(at(a, b, c, 6), k3, 1);
    if (b != c) {
      set(at(a, c, b, 0), k1, 1);
      set(at(a, c, b, 1), k2, -1);
      add(at(a, c, b, 3), k3, 1);
      add(at(a, c, b, 5), k3, 1);
      add(at(a, c, b, 6), k3, 1);
    }
    set(at(c, a, b, 2), k2, 1);
    add(at(c, a, b, 3), k3, 1);
    add(at(c, a, b, 5), k3, -1);
    add(at(c, a, b, 6), k3, 1);
    if (b != c) {
      set(at(b, a, c, 2), k2, 1);
      add(at(b, a, c, 3), k3, 1);
      add(at(b, a, c, 5), k3, -1);
      add(at(b, a, c, 6), k3, 1);
    }
    set(at(b, c, a, 4), k2, 2);
    add(at(b, c, a, 6), k3, 4);
    if (b != c) {
      set(at(c, b, a, 4), k2, 2);
      add(at(c, b, a, 6), k3, 4);
    }
  }
}

static std::vector<int> sym_offsets(int nL, int nM, int nN) {
  std::vector<int> o;
  for (int mx = 0; mx < nL; ++mx)
    for (int my = 0; my < nM; ++my)
      for (int mz = 0; mz <= my; ++mz) {
        o.push_back(mx);
        o.push_back(my);
        o.push_back(mz);
      }
  (void)nN;
  return o;
}

// Builds fN_all (column-major (2L, 2M, 2N, 7), device, caller-allocated) and st (3 complex, host).
void circulant_tensor_device(int L, int M, int N, double dx, double2* fN_dev, double2 st_out[3], cudaStream_t st) {
  VH_REQUIRE(L >= 2 && M >= 2 && N >= 2, ERR_UNSUPPORTED,
             "grids thinner than 2 voxels need the singular-integral path of the reference");
  const int64_t PG = (int64_t)L * M * N;
  double2* G = nullptr;
  VH_CUDA_TRY(cudaMalloc(&G, 7 * PG * sizeof(double2)));
  try {
    // far interactions, 3-point rule on every offset (lse_generate_circulant_tensor.m:56-74)
    const DiffTable t3 = diff_table(3, dx / 2);
    k_volume_volume<<<(unsigned)std::min<int64_t>(65535, ceil_div(PG, 128)), 128, 0, st>>>(t3, dx, L, M, N, L, M, N, G);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    // the block of offsets < 5 in every axis is rewritten by the medium and near terms
    const int nL = std::min(5, L), nM = std::min(5, M), nN = std::min(5, N);
    std::vector<double2> G5((size_t)nL * nM * nN * 7);
    auto copy_block = [&](bool to_host) {
      for (int k = 0; k < 7; ++k)
        for (int z = 0; z < nN; ++z)
          for (int y = 0; y < nM; ++y) {
            double2* dev = G + (int64_t)L * (y + (int64_t)M * z) + k * PG;
            double2* hst = G5.data() + (size_t)nL * (y + (size_t)nM * (z + (size_t)nN * k));
            if (to_host) VH_CUDA_TRY(cudaMemcpyAsync(hst, dev, nL * sizeof(double2), cudaMemcpyDeviceToHost, st));
            else VH_CUDA_TRY(cudaMemcpyAsync(dev, hst, nL * sizeof(double2), cudaMemcpyHostToDevice, st));
          }
      VH_CUDA_TRY(cudaStreamSynchronize(st));
    };
    const DiffTable t5 = diff_table(5, dx / 2);
    if (nL != nM || nL != nN) {
      // medium interactions without symmetry (:92-107): 5-point rule on the whole block
      double2* Gm = nullptr;
      VH_CUDA_TRY(cudaMalloc(&Gm, 7 * (int64_t)nL * nM * nN * sizeof(double2)));
      k_volume_volume<<<64, 128, 0, st>>>(t5, dx, nL, nM, nN, nL, nM, nN, Gm);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      VH_CUDA_TRY(cudaMemcpyAsync(G5.data(), Gm, G5.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
      cudaFree(Gm);
    } else {
      // medium interactions exploiting symmetry (:146-306)
      copy_block(true);
      const std::vector<int> offs = sym_offsets(nL, nM, nN);
      const int no = (int)offs.size() / 3;
      int* d_offs = nullptr;
      double2* d_K = nullptr;
      VH_CUDA_TRY(cudaMalloc(&d_offs, offs.size() * sizeof(int)));
      VH_CUDA_TRY(cudaMalloc(&d_K, 3 * no * sizeof(double2)));
      VH_CUDA_TRY(cudaMemcpyAsync(d_offs, offs.data(), offs.size() * sizeof(int), cudaMemcpyHostToDevice, st));
      k_volume_volume_sym<<<no, 256, 0, st>>>(t5, dx, d_offs, d_K);
      count_launch();
      VH_CUDA_TRY(cudaGetLastError());
      std::vector<double2> K(3 * no);
      VH_CUDA_TRY(cudaMemcpyAsync(K.data(), d_K, K.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
      VH_CUDA_TRY(cudaStreamSynchronize(st));
      cudaFree(d_offs);
      cudaFree(d_K);
      std::fill(G5.begin(), G5.end(), make_double2(0.0, 0.0));
      scatter_sym(G5, nL, nM, nN, offs, K);
    }
    // near interactions from the 1 mm table scaled by (dx/1e-3)^{5,6,7} (:328-492)
    {
      const int Ls = std::min(2, L), Ms = std::min(2, M), Ns = std::min(2, N);
      VH_REQUIRE(Ls == Ms && Ls == Ns, ERR_UNSUPPORTED, "near-field table needs at least 2 voxels per axis");
      const std::vector<int> offs = sym_offsets(Ls, Ms, Ns);
      const double s = dx / 1e-3;
      const double sc[3] = {std::pow(s, 5), std::pow(s, 6), std::pow(s, 7)};
      std::vector<double2> K(offs.size());
      for (size_t e = 0; e < offs.size() / 3; ++e)
        for (int i = 0; i < 3; ++i) K[3 * e + i] = make_double2(kNear1mm[e][i][0] * sc[i], kNear1mm[e][i][1] * sc[i]);
      for (int k = 0; k < 7; ++k)
        for (int z = 0; z < Ns; ++z)
          for (int y = 0; y < Ms; ++y)
            for (int x = 0; x < Ls; ++x) G5[x + nL * (y + nM * (z + (size_t)nN * k))] = make_double2(0.0, 0.0);
      scatter_sym(G5, nL, nM, nN, offs, K);
    }
    copy_block(false);
    k_normalise<<<1024, 256, 0, st>>>(G, PG, dx);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    // self terms for the preconditioner (:772), after normalisation
    double2 s3[3];
    for (int i = 0; i < 3; ++i) {
      const int k = i == 0 ? 0 : (i == 1 ? 3 : 6);
      VH_CUDA_TRY(cudaMemcpyAsync(&s3[i], G + k * PG, sizeof(double2), cudaMemcpyDeviceToHost, st));
    }
    k_embed<<<2048, 256, 0, st>>>(G, L, M, N, fN_dev);
    count_launch();
    VH_CUDA_TRY(cudaGetLastError());
    VH_CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < 3; ++i) st_out[i] = s3[i];
    // fft_operator.m: 3-D FFT of each component
    fft3d_forward_inplace(fN_dev, 2 * L, 2 * M, 2 * N, 7, st);
  } catch (...) {
    cudaFree(G);
    throw;
  }
  cudaFree(G);
}

// ---------------------------------------------------------------------------- panel numbering
// lse_generate_panelIDs.m:25-172: x panels scan x fastest (then y, z), y panels y fastest (then z, x),
// z panels z fastest (then x, y); consecutive non-empty voxels along the scanned axis share a panel.
void panel_ids(int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t* apid, int64_t* num_nodes) {
  const int64_t lmn = (int64_t)L * M * N;
  std::vector<int64_t> vnum(lmn, -1);
  for (int64_t v = 0; v < nv; ++v) {
    const int64_t li = idxS[v] - 1;
    VH_REQUIRE(li >= 0 && li < lmn && (v == 0 || idxS[v] > idxS[v - 1]), ERR_BAD_ARG,
               "idxS must be strictly increasing 1-based indices into the grid");
    vnum[li] = v;
  }
  auto lin = [&](int x, int y, int z) { return x + (int64_t)L * (y + (int64_t)M * z); };
  int64_t offset = 0;
  const int dims[3] = {L, M, N};
  for (int axis = 0; axis < 3; ++axis) {
    // loop order: the two other axes in the reference's nesting, the scanned axis innermost
    const int o1 = axis == 0 ? 2 : (axis == 1 ? 0 : 1);     // outer
    const int o2 = axis == 0 ? 1 : (axis == 1 ? 2 : 0);     // middle
    int64_t ind = 1;
    int c[3];
    for (c[o1] = 0; c[o1] < dims[o1]; ++c[o1])
      for (c[o2] = 0; c[o2] < dims[o2]; ++c[o2])
        for (c[axis] = 0; c[axis] < dims[axis]; ++c[axis]) {
          const int64_t v = vnum[lin(c[0], c[1], c[2])];
          if (v < 0) continue;
          bool next_empty = c[axis] + 1 >= dims[axis];
          if (!next_empty) {
            int d[3] = {c[0], c[1], c[2]};
            d[axis] += 1;
            next_empty = vnum[lin(d[0], d[1], d[2])] < 0;
          }
          apid[v + nv * (2 * axis)] = offset + ind;
          apid[v + nv * (2 * axis + 1)] = offset + ind + 1;
          ind += 1;
          if (next_empty) ind += 1;
        }
    int64_t np = 0;
    for (int64_t v = 0; v < nv; ++v) np = std::max(np, apid[v + nv * (2 * axis + 1)] - offset);
    offset += np;
  }
  *num_nodes = offset;
}

}  // namespace vh

using namespace vh;

extern "C" {

vh_status vh_panel_ids(int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t* all_panels_ids,
                       int64_t* num_nodes) {
  try {
    VH_REQUIRE(L >= 1 && M >= 1 && N >= 1 && nv >= 0 && (nv == 0 || (idxS && all_panels_ids)) && num_nodes,
               ERR_BAD_ARG, "bad arguments");
    panel_ids(L, M, N, nv, idxS, all_panels_ids, num_nodes);
    return VH_OK;
  } catch (const Error& e) {
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {
    return VH_ERR_OOM;
  }
}

// lse_compute_Ae_matrix.m:205-264: columns Jx, Jy, Jz, J2D, J3D of every voxel; 16 nv entries.
vh_status vh_incidence(int64_t nv, const int64_t* all_panels_ids, int64_t* Ae_jc, int64_t* Ae_ir, double* Ae_pr) {
  if (nv < 0 || (nv > 0 && (!all_panels_ids || !Ae_jc || !Ae_ir || !Ae_pr))) return VH_ERR_BAD_ARG;
  static const double coef[5][6] = {{-1, 1, 0, 0, 0, 0},          {0, 0, -1, 1, 0, 0},        {0, 0, 0, 0, -1, 1},
                                    {0.5, 0.5, -0.5, -0.5, 0, 0}, {0.5, 0.5, 0.5, 0.5, -1, -1}};
  int64_t k = 0;
  Ae_jc[0] = 0;
  for (int c = 0; c < 5; ++c)
    for (int64_t v = 0; v < nv; ++v) {
      for (int p = 0; p < 6; ++p)
        if (coef[c][p] != 0.0) {
          Ae_ir[k] = all_panels_ids[v + nv * p] - 1;   // panel ids increase with p: rows stay sorted
          Ae_pr[k] = coef[c][p];
          ++k;
        }
      Ae_jc[c * nv + v + 1] = k;
    }
  return VH_OK;
}

vh_status vh_circulant_tensor(vh_ctx* ctx, int L, int M, int N, double dx, double* fN_all, double* st_sparse_precon) {
  if (!ctx) return VH_ERR_BAD_ARG;
  try {
    VH_CUDA_TRY(cudaSetDevice(ctx->device));
    const int64_t P = 8LL * L * M * N;
    double2* d = nullptr;
    VH_CUDA_TRY(cudaMalloc(&d, 7 * P * sizeof(double2)));
    double2 s3[3];
    try {
      circulant_tensor_device(L, M, N, dx, d, s3, ctx->stream);
      if (fN_all) VH_CUDA_TRY(cudaMemcpyAsync(fN_all, d, 7 * P * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
      VH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      cudaFree(d);
      throw;
    }
    cudaFree(d);
    if (st_sparse_precon)
      for (int i = 0; i < 3; ++i) {
        st_sparse_precon[2 * i] = s3[i].x;
        st_sparse_precon[2 * i + 1] = s3[i].y;
      }
    return VH_OK;
  } catch (const Error& e) {
    ctx->last_error = e.msg;
    return (vh_status)e.st;
  } catch (const std::bad_alloc&) {
    return VH_ERR_OOM;
  }
}

}  // extern "C"
