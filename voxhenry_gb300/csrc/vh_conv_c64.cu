// The complex64 instantiation of the FFT convolution passes (the inner matvec of the mixed-precision
// solver).
#include "vh_conv_passes.cuh"

namespace vh {

void conv_apply_c64(ConvPlan& p, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy, const double2* scale,
                    const double2* zdiag, int64_t zstride, cudaStream_t st) {
  conv_apply_t<float>(p, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
}

}  // namespace vh
