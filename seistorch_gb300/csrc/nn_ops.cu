// Memory-bound helper kernels of the learned preconditioner (layouts,
// pooling, upsampling, small convolutions, optimiser): plain SIMT code.
#include <cuda_bf16.h>
#include <stdint.h>

#include "sgb_common.cuh"

namespace sgb {
namespace nn {
namespace {

// out[k][n][c][y][x] = in[n][y][x - 1 + k][coff + c] (k over copies; with one
// copy k = 1, the plain transpose).  One thread per (n, c, y, x).
__global__ void to_chw_kernel(int n, int h, int w, int c, int cstride, int coff, const __nv_bfloat16* in,
                              int copies, __nv_bfloat16* out) {
  const long long total = (long long)n * c * h * w;
  const long long plane = total;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % w);
    long long r = i / w;
    const int y = (int)(r % h);
    r /= h;
    const int ch = (int)(r % c);
    const int b = (int)(r / c);
    for (int k = 0; k < copies; ++k) {
      const int shift = copies == 1 ? 0 : k - 1;
      const int xs = x + shift;
      __nv_bfloat16 v = __float2bfloat16_rn(0.f);
      if (xs >= 0 && xs < w) v = in[(((long long)b * h + y) * w + xs) * cstride + coff + ch];
      out[k * plane + i] = v;
    }
  }
}

int blocks_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

}  // namespace

cudaError_t launch_to_chw(int n, int h, int w, int c, int cstride, int coff, const __nv_bfloat16* x, int copies,
                          __nv_bfloat16* out, cudaStream_t s) {
  const long long total = (long long)n * c * h * w;
  to_chw_kernel<<<blocks_for(total), 256, 0, s>>>(n, h, w, c, cstride, coff, x, copies, out);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace sgb
