// Circulant-embedded Toeplitz convolution of the VIE operator (the FFT part of
// lse_matvect_mult.m:34-128) for a batch of right-hand sides.
#pragma once
#include <vector>

#include "vh_common.cuh"
#include "vh_fft.cuh"

namespace vh {

// PREC_DF: complex128 storage and FP64 x/y transforms, the z-pass (transform, tensor products,
// inverse) in double-float arithmetic on the FP32 pipes (~48 significant bits)
enum Prec { PREC_FP64 = 0, PREC_FP32 = 1, PREC_DF = 2 };

// Factor n into the radices the FFT supports; false if n has another prime factor.
bool fft_factor(int n, FftDesc& d);

// Launch choices of the FFT convolution at one precision, set by the autotuner (vh_conv_tune) or from
// its cache (vh_conv_set_tuning): the y-pass (0 automatic = the register pass where Y is 256, 512 or
// 1024, over 64-byte row segments for complex64; 1 the register pass over 128-byte row segments; 2 the
// shared-memory Stockham pass; 3 the register pass over 64-byte row segments), the z-pass (z_variant)
// and the
// right-hand sides per launch sequence (0: the whole batch; else chunks of at most max_rhs, which
// keeps the spectra of a chunk smaller at the price of reading the tensor once per chunk).
struct ConvTuning {
  int y_variant = 0;
  int max_rhs = 0;
  // x passes (complex64): 0 automatic = 1 where X is 256, 512 or 1024; 1 one warp per line; 2 the
  // shared-memory passes
  int x_variant = 0;
  int z_variant = 0;   // 0 automatic = 3 for complex64 where nz <= kZtoepMaxRows, else 1; 1 the two-lane
                       // register z-pass; 2 one thread per column (Z <= 32); 3 (complex64, double-float)
                       // the direct Toeplitz convolution along z (nz <= kZtoepMaxRows)
};

constexpr int kZtoepMaxRows = 16;

struct ConvPlan {
  int L = 0, M = 0, N = 0;   // voxel grid
  int X = 0, Y = 0, Z = 0;   // padded grid (2L, 2M, 2N)
  int64_t nv = 0;            // non-empty voxels
  // bounding box of the voxels in y and z: the x-passes run over lines y0 <= y < y0+ny,
  // z0 <= z < z0+nz only, and the y- and z-FFTs load and keep only those rows (every other line
  // of the zero-padded operands is zero, and only voxel rows of the result are used)
  int y0 = 0, ny = 0, z0 = 0, nz = 0;
  double dx = 0;
  FftDesc fx{}, fy{}, fz{};
  int32_t* vmap = nullptr;   // (L*M*N) voxel -> compact index or -1, column-major
  // internal tensor spectrum, layout [ky][kz][k][kx], already divided by X*Y*Z
  double2* tens64 = nullptr;
  float2* tens32 = nullptr;
  // complex64 products with a real/imaginary tensor: every component of the spectrum is real (0, 3,
  // 5, 6) or imaginary (1, 2, 4) -- the kernel is even or odd along each axis -- so tens32ri holds
  // one float per component (the real or the imaginary part, layout as tens32); set when the
  // spectrum was checked to be of that form to within 1e-9 of each component's magnitude
  float* tens32ri = nullptr;
  bool ri = false;            // the spectrum has the real/imaginary form above (checked at creation)
  void* tensdf = nullptr;     // double-float real/imaginary tensor (one pair of floats per component,
                              // layout as tens32ri), built on first PREC_DF use when ri holds
  // z_variant 3: h_k(kx, ky, d) = sum_kz S_k e^{+2 pi i kz d / Z} for 0 <= d < nz, one float per value
  // (real, or the imaginary part for components 1 and 2), layout [ky][k][d][kx], followed by the
  // low floats of the same values as double-float pairs; built on first use
  float* tensz = nullptr;
  int ztoep_state = 0;        // 0 not built, 1 built, -1 not available (nz too large or form check failed)
  void* twdf = nullptr;       // double-float z twiddles
  void* twxdf = nullptr;      // double-float x and y twiddles
  void* twydf = nullptr;
  double2* tw64[3] = {nullptr, nullptr, nullptr};
  float2* tw32[3] = {nullptr, nullptr, nullptr};
  // scratch: A (5 * nz * ny * X per RHS) and Bf (5 * nz * Y * X per RHS), in bytes
  void* scratchA = nullptr;
  void* scratchB = nullptr;
  size_t scratch_bytes_A = 0, scratch_bytes_B = 0;
  ConvTuning tune[3];          // per Prec
  int y_variant_now = 0;       // the x-, y- and z-passes of the launch sequence being issued (ConvTuning)
  int z_variant_now = 0;
  int x_variant_now = 0;

  int64_t points() const { return (int64_t)X * Y * Z; }
  int64_t lmn() const { return (int64_t)L * M * N; }
};

// Builds the plan. `fN_all` is the reference's circulant tensor spectrum (complex,
// column-major (2L, 2M, 2N, 7)), on the DEVICE. `idxS` (1-based, sorted) on the HOST.
void conv_plan_create(ConvPlan& p, int L, int M, int N, double dx, const double2* fN_all_dev, int64_t nv,
                      const int64_t* idxS_host, bool want32, cudaStream_t st);
void conv_plan_destroy(ConvPlan& p);
// Ensures the scratch buffers hold `B` right-hand sides at precision `prec`.
void conv_plan_reserve(ConvPlan& p, int B, Prec prec);

// y_J[b] = scale[b] * conv(x_J[b]) + (c_k / dx) * zdiag[b] * x_J[b]  for the 5*nv current unknowns.
//   x, y      : device, complex double, RHS b at x + b*ldx (only the first 5*nv entries used)
//   scale     : device, B complex (j omega mu per RHS; 1 for the drop-in form)
//   zdiag     : device, complex per voxel, RHS b uses zdiag + b*zstride (zstride 0 = shared)
void conv_apply(ConvPlan& p, Prec prec, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st);

// Bytes of FFT scratch one right-hand side needs at precision `prec`: A (5 nz ny X complex values)
// and Bf (5 nz Y X complex values), at most 30 L M N values in all.
void conv_scratch_bytes(const ConvPlan& p, Prec prec, size_t& a_per_rhs, size_t& b_per_rhs);

// conv_apply with caller-provided scratch (scratchA: B * a_per_rhs bytes, scratchB: B * b_per_rhs
// bytes, both 16-byte aligned), for callers that cannot allocate device memory: it reserves nothing
// and allocates nothing.  Every scratch element a pass reads was written by an earlier pass, so the
// scratch needs no clearing.
void conv_apply_scratch(const ConvPlan& p, Prec prec, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                        const double2* scale, const double2* zdiag, int64_t zstride, void* scratchA, void* scratchB,
                        cudaStream_t st);

// The z-pass of z_variant 3 (complex64): builds the Toeplitz table on first call (false when the
// geometry does not take it), and the pass itself on Bf (false when the table is not built).
bool ztoep_build(ConvPlan& p, cudaStream_t st);
bool zpass_toep(const ConvPlan& p, float2* Bf, int B, cudaStream_t st);
// The x passes of x variant 1 (complex64): one warp per line for X = 256, 512, 1024
// (vh_conv_xwarp.cu); false where X is another length.
bool xpass_warp_ok(const ConvPlan& p);
bool xpass_warp_fwd(const ConvPlan& p, int B, const double2* x, int64_t ldx, float2* A, cudaStream_t st);
bool xpass_warp_inv(const ConvPlan& p, int B, const float2* A, const double2* x, int64_t ldx, double2* y, int64_t ldy,
                    const double2* scale, const double2* zdiag, int64_t zstride, cudaStream_t st);
// the same in double-float arithmetic on pair storage (PREC_DF)
struct dcomplex;
bool zpass_toep_df(const ConvPlan& p, dcomplex* Bf, int B, cudaStream_t st);
// The Toeplitz passes stage their inputs with the copy engine and wait for the copies a bounded number
// of polls; a pass that gave up wrote NaN and raised a device flag.  Reads and clears that flag (one
// per device process, shared by all contexts), after the work on `st` is done.
bool ztoep_take_stall(cudaStream_t st);

// In-place forward 3-D FFT of `batch` column-major X x Y x Z complex arrays (device).
void fft3d_forward_inplace(double2* data, int X, int Y, int Z, int batch, cudaStream_t st);

// Circulant tensor spectrum fN_all (column-major (2L, 2M, 2N, 7), device, caller-allocated) and
// the three self terms st (host) of lse_generate_circulant_tensor(dx, 1, L, M, N, 0).
void circulant_tensor_device(int L, int M, int N, double dx, double2* fN_dev, double2 st_out[3], cudaStream_t st);

}  // namespace vh
