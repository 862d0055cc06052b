// The register z-pass of the double-float FFT convolution (pairs of floats in storage and arithmetic,
// the real/imaginary tensor), in its own translation unit so that it compiles beside the x and y
// passes.
#include "vh_conv_passes.cuh"

namespace vh {

bool zpass_df(int z_variant, int Z, int nz, dcomplex* Bf, const dfloat* tens_ri, int Y, int X, int B,
              const dcomplex* tw, cudaStream_t st) {
  return zpass_any<dfloat>(z_variant, Z, nz, Bf, tens_ri, Y, X, B, tw, st);
}

}  // namespace vh
