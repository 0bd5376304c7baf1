// Argument block of the tcgen05 GEMM (nn_gemm.cu) behind the learned
// preconditioner's convolutions.
#pragma once

#include <cuda_bf16.h>

namespace sgb {
namespace nn {

enum { MODE_CONV = 0, MODE_WGRAD = 1 };

struct GemmArgs {
  int mode;
  int N, H, W, Cin, Cout;
  // CONV: output tile = TH rows x TW columns of one image (TH * TW = 128)
  int TW, TH, tiles_x, tiles_y;
  int nchunk;       // input channels / channels per K step
  int kiters;       // K steps (CONV: 9 * nchunk; WGRAD: N * H * wchunks)
  int wchunks;      // WGRAD: W / 64
  int k_per_split;  // WGRAD: K steps per CTA
  // CONV epilogue: v = acc (+ bias) (relu) (* [mask > 0]); stored at
  // out[pixel * out_cstride + out_coff + co]
  const float* bias;
  int relu;
  const __nv_bfloat16* mask;
  int mask_cstride;
  __nv_bfloat16* out_bf16;
  float* out_f32;  // CONV: optional fp32 copy; WGRAD: dW [Cout][Cin][3][3] (accumulated)
  int out_cstride, out_coff;
  int* status;
  // logical tile grid (x, y, z) of the persistent kernel: tile t is
  // (t % gx, (t / gx) % gy, t / (gx * gy))
  int gx, gy, gz;
};

}  // namespace nn
}  // namespace sgb
