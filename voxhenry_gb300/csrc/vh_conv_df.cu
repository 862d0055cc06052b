// The double-float instantiation of the FFT convolution passes: the VH_PREC_DF product (the
// refinement residual of the mixed-precision solver), its spectra kept as pairs of floats between
// the passes.
#include "vh_conv_passes.cuh"

namespace vh {

void conv_apply_df(ConvPlan& p, int B, const double2* x, int64_t ldx, double2* y, int64_t ldy, const double2* scale,
                   const double2* zdiag, int64_t zstride, cudaStream_t st) {
  conv_apply_t<dfloat>(p, B, x, ldx, y, ldy, scale, zdiag, zstride, st);
}

}  // namespace vh
