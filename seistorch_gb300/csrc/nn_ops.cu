// Memory-bound helper kernels of the learned preconditioner (layouts,
// pooling, upsampling, the 2-channel input and 1-channel output
// convolutions, weight packing, optimiser, loss): plain SIMT code.  The
// heavy 3x3 convolutions run on the tensor cores (nn_gemm.cu).
//
// Activations are bf16 NHWC; a tensor may be a channel slice [coff, coff+c)
// of a wider one with cstride channels per pixel.  Channel counts, strides
// and offsets are multiples of 8 (16-byte channel vectors).
#include <cuda_bf16.h>
#include <stdint.h>

#include "sgb_common.cuh"

namespace sgb {
namespace nn {
namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ float ld(const bf16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ bf16 st(float v) { return __float2bfloat16_rn(v); }

int blocks_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b > 152 * 32 ? 152 * 32 : (b < 1 ? 1 : b));
}

// 8 bf16 channels moved as one 16-byte vector (little-endian pairs: the
// lower half of each 32-bit word is the even channel).
__device__ __forceinline__ void unpack8(const uint4& u, float (&f)[8]) {
  const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    f[2 * k] = __uint_as_float(w[k] << 16);
    f[2 * k + 1] = __uint_as_float(w[k] & 0xffff0000u);
  }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
  unsigned w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
    w[k] = *reinterpret_cast<const unsigned*>(&h2);
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ __forceinline__ uint4 ld8(const bf16* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }
__device__ __forceinline__ void st8(bf16* p, const uint4& v) { *reinterpret_cast<uint4*>(p) = v; }

#define GRID_STRIDE(i, total) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (total); i += (long long)gridDim.x * blockDim.x)

// out[k][n][c][y][x] = in[n][y][x - 1 + k][coff + c] (one copy: k = 1).
// A block moves a tile of 32 columns (plus the one-column halo the shifted
// copies read) of one image row through shared memory: 16-byte reads of
// the channel vectors, 64-byte coalesced rows of the channel-major output.
constexpr int TCHW_X = 32;
__global__ void to_chw_kernel(int n, int h, int w, int c, int cstride, int coff, const bf16* in, int copies,
                              bf16* out) {
  extern __shared__ __align__(16) bf16 tile[];  // [TCHW_X + 2][c]
  const int row = blockIdx.y;  // b * h + y
  const int x0 = blockIdx.x * TCHW_X;
  const int cv = c / 8;
  for (int q = threadIdx.x; q < (TCHW_X + 2) * cv; q += blockDim.x) {
    const int px = q / cv, k8 = (q % cv) * 8;
    const int x = x0 - 1 + px;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (x >= 0 && x < w) v = ld8(in + ((long long)row * w + x) * cstride + coff + k8);
    st8(tile + px * c + k8, v);
  }
  __syncthreads();
  const long long plane = (long long)n * c * h * w;
  const int b = row / h, y = row % h;
  for (int q = threadIdx.x; q < copies * c * TCHW_X; q += blockDim.x) {
    const int xx = q % TCHW_X;
    const int ch = (q / TCHW_X) % c;
    const int k = q / (TCHW_X * c);
    const int x = x0 + xx;
    if (x >= w) continue;
    const int shift = copies == 1 ? 0 : k - 1;
    out[k * plane + (((long long)b * c + ch) * h + y) * w + x] = tile[(xx + 1 + shift) * c + ch];
  }
}

// Input convolution: 2 fp32 channels [n][2][h][w] -> c bf16 channels (ReLU).
template <bool SMEM_W>
__global__ void conv_in_fwd_kernel(int n, int h, int w, int c, const float* in, const float* W, const float* b,
                                   bf16* out, int cstride, int coff) {
  // the weights (18 per output channel) and biases: staged once per block
  // where they fit, read by every thread of the block as broadcasts
  extern __shared__ float cin_w[];
  if (SMEM_W) {
    for (int k = threadIdx.x; k < 19 * c; k += blockDim.x) cin_w[k] = k < 18 * c ? W[k] : b[k - 18 * c];
    __syncthreads();
  }
  const float* Wp = SMEM_W ? cin_w : W;
  const float* bp = SMEM_W ? cin_w + 18 * c : b;
  const long long total = (long long)n * h * w;
  GRID_STRIDE(i, total) {
    const int x = (int)(i % w);
    const int y = (int)((i / w) % h);
    const int bb = (int)(i / ((long long)w * h));
    float v[18];
    for (int ci = 0; ci < 2; ++ci)
      for (int ky = 0; ky < 3; ++ky)
        for (int kx = 0; kx < 3; ++kx) {
          const int yy = y - 1 + ky, xx = x - 1 + kx;
          v[ci * 9 + ky * 3 + kx] =
              (yy >= 0 && yy < h && xx >= 0 && xx < w) ? in[(((long long)bb * 2 + ci) * h + yy) * w + xx] : 0.f;
        }
    for (int c8 = 0; c8 < c; c8 += 8) {
      float o[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int co = c8 + j;
        float a = bp[co];
#pragma unroll
        for (int k = 0; k < 18; ++k) a = fmaf(Wp[co * 18 + k], v[k], a);
        o[j] = a > 0.f ? a : 0.f;
      }
      st8(out + i * cstride + coff + c8, pack8(o));
    }
  }
}

// Weight / bias gradient of the input convolution: block (co, split).
__global__ void conv_in_wgrad_kernel(int n, int h, int w, int c, const float* in, const bf16* dy, int dy_cstride,
                                     float* dW, float* db) {
  const int co = blockIdx.y;
  const long long total = (long long)n * h * w;
  float acc[19];
  for (int k = 0; k < 19; ++k) acc[k] = 0.f;
  GRID_STRIDE(i, total) {
    const float g = ld(dy + i * dy_cstride + co);
    if (g == 0.f) continue;
    const int x = (int)(i % w);
    const int y = (int)((i / w) % h);
    const int bb = (int)(i / ((long long)w * h));
    for (int ci = 0; ci < 2; ++ci)
      for (int ky = 0; ky < 3; ++ky)
        for (int kx = 0; kx < 3; ++kx) {
          const int yy = y - 1 + ky, xx = x - 1 + kx;
          if (yy >= 0 && yy < h && xx >= 0 && xx < w)
            acc[ci * 9 + ky * 3 + kx] += g * in[(((long long)bb * 2 + ci) * h + yy) * w + xx];
        }
    acc[18] += g;
  }
  for (int k = 0; k < 19; ++k) {
    float v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) {
      if (k < 18)
        atomicAdd(dW + co * 18 + k, v);
      else
        atomicAdd(db + co, v);
    }
  }
}

// Output convolution: c bf16 channels -> 1 fp32 channel (linear).
__global__ void conv_out_fwd_kernel(int n, int h, int w, int c, const bf16* in, int cstride, const float* W,
                                    const float* b, float* out) {
  const long long total = (long long)n * h * w;
  GRID_STRIDE(i, total) {
    const int x = (int)(i % w);
    const int y = (int)((i / w) % h);
    const int bb = (int)(i / ((long long)w * h));
    float a = b[0];
    for (int ky = 0; ky < 3; ++ky)
      for (int kx = 0; kx < 3; ++kx) {
        const int yy = y - 1 + ky, xx = x - 1 + kx;
        if (yy < 0 || yy >= h || xx < 0 || xx >= w) continue;
        const bf16* p = in + (((long long)bb * h + yy) * w + xx) * cstride;
        for (int c8 = 0; c8 < c; c8 += 8) {
          float f[8];
          unpack8(ld8(p + c8), f);
#pragma unroll
          for (int j = 0; j < 8; ++j) a = fmaf(W[(c8 + j) * 9 + ky * 3 + kx], f[j], a);
        }
      }
    out[i] = a;
  }
}

// The same convolution for c <= 64 from shared memory: a block of 256
// threads takes 256 pixels of one image row, stages the three input rows
// (258 pixels with the halo, c channels, 16-byte vectors) and the weights
// (tap-major) once, and each thread sums its pixel's 9 taps from there.  A
// thread walks its pixel's channel vectors starting at (lane mod c/8), so
// that the 8 threads of a 16-byte access phase hit distinct banks.
constexpr int COUT_TX = 256;
template <int CV>  // channel vectors per pixel (c = 8 CV)
__global__ void __launch_bounds__(COUT_TX) conv_out_tile_kernel(int n, int h, int w, const bf16* in, int cstride,
                                                                 const float* W, const float* b, float* out) {
  extern __shared__ __align__(16) unsigned char cout_smem[];
  constexpr int cv = CV, c = 8 * CV, cols = COUT_TX + 2;
  uint4* srow = reinterpret_cast<uint4*>(cout_smem);  // [3][cols][cv]
  float* ws = reinterpret_cast<float*>(srow + 3 * cols * cv);  // [9][c]
  const int ntx = (w + COUT_TX - 1) / COUT_TX;
  const int xt = blockIdx.x % ntx;
  const long long ry = blockIdx.x / ntx;
  const int y = (int)(ry % h), bb = (int)(ry / h);
  const int x0 = xt * COUT_TX;
  for (int k = threadIdx.x; k < 9 * c; k += COUT_TX) {
    const int tap = k / c, ci = k - tap * c;
    ws[k] = W[ci * 9 + tap];
  }
  // eight vectors per thread in flight at a time: loads first, then stores
  const int nvec = 3 * cols * cv;
  for (int k0 = threadIdx.x; k0 < nvec; k0 += 8 * COUT_TX) {
    uint4 q[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = k0 + u * COUT_TX;
      q[u] = make_uint4(0u, 0u, 0u, 0u);
      if (k < nvec) {
        const int v = k % cv, rc = k / cv;
        const int col = rc % cols, r = rc / cols;
        const int yy = y - 1 + r, xx = x0 - 1 + col;
        if (yy >= 0 && yy < h && xx >= 0 && xx < w) q[u] = ld8(in + (((long long)bb * h + yy) * w + xx) * cstride + 8 * v);
      }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k0 + u * COUT_TX < nvec) srow[k0 + u * COUT_TX] = q[u];
  }
  __syncthreads();
  const int t = threadIdx.x, x = x0 + t;
  if (x >= w) return;
  float acc[4] = {b[0], 0.f, 0.f, 0.f};  // four partial sums: short FMA chains
#pragma unroll
  for (int tap = 0; tap < 9; ++tap) {
    const int ky = tap / 3, kx = tap - 3 * ky;
    const uint4* px = srow + (ky * cols + t + kx) * cv;
    const float* wt = ws + tap * c;
#pragma unroll
    for (int vv = 0; vv < cv; ++vv) {
      const int v = (vv + t) & (cv - 1);
      float f[8];
      unpack8(px[v], f);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j & 3] = fmaf(wt[8 * v + j], f[j], acc[j & 3]);
    }
  }
  out[((long long)bb * h + y) * w + x] = (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// Data gradient of the output convolution, times [act > 0] (the ReLU of the
// layer that produced its input): dx[p][ci] = sum_tap W[ci][tap] g[p - off].
__global__ void conv_out_dgrad_kernel(int n, int h, int w, int c, const float* g, const float* W, const bf16* act,
                                      int act_cstride, bf16* dx) {
  const long long total = (long long)n * h * w;
  GRID_STRIDE(i, total) {
    const int x = (int)(i % w);
    const int y = (int)((i / w) % h);
    const int bb = (int)(i / ((long long)w * h));
    float gv[9];
    for (int ky = 0; ky < 3; ++ky)
      for (int kx = 0; kx < 3; ++kx) {
        // output pixel (y + 1 - ky, x + 1 - kx) reads this pixel through tap (ky, kx)
        const int yy = y + 1 - ky, xx = x + 1 - kx;
        gv[ky * 3 + kx] = (yy >= 0 && yy < h && xx >= 0 && xx < w) ? g[((long long)bb * h + yy) * w + xx] : 0.f;
      }
    for (int c8 = 0; c8 < c; c8 += 8) {
      float o[8], m[8];
      unpack8(ld8(act + i * act_cstride + c8), m);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float a = 0.f;
        for (int k = 0; k < 9; ++k) a = fmaf(W[(c8 + j) * 9 + k], gv[k], a);
        o[j] = m[j] > 0.f ? a : 0.f;
      }
      st8(dx + i * c + c8, pack8(o));
    }
  }
}

// Weight / bias gradient of the output convolution: block (ci, split).
__global__ void conv_out_wgrad_kernel(int n, int h, int w, int c, const float* g, const bf16* in, int cstride,
                                      float* dW, float* db) {
  const int ci = blockIdx.y;
  const long long total = (long long)n * h * w;
  float acc[10];
  for (int k = 0; k < 10; ++k) acc[k] = 0.f;
  GRID_STRIDE(i, total) {
    const float gv = g[i];
    const int x = (int)(i % w);
    const int y = (int)((i / w) % h);
    const int bb = (int)(i / ((long long)w * h));
    for (int ky = 0; ky < 3; ++ky)
      for (int kx = 0; kx < 3; ++kx) {
        const int yy = y - 1 + ky, xx = x - 1 + kx;
        if (yy >= 0 && yy < h && xx >= 0 && xx < w)
          acc[ky * 3 + kx] += gv * ld(in + (((long long)bb * h + yy) * w + xx) * cstride + ci);
      }
    acc[9] += gv;
  }
  for (int k = 0; k < 10; ++k) {
    float v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) {
      if (k < 9)
        atomicAdd(dW + ci * 9 + k, v);
      else if (ci == 0)
        atomicAdd(db, v);
    }
  }
}

// 2x2 average pooling; h, w are the input dims; 8 channels per thread.
__global__ void pool2_kernel(int n, int h, int w, int c, const bf16* in, int cs_in, int coff_in, bf16* out) {
  const int ho = h / 2, wo = w / 2, cv = c / 8;
  const long long total = (long long)n * ho * wo * cv;
  GRID_STRIDE(i, total) {
    const int c8 = (int)(i % cv) * 8;
    long long r = i / cv;
    const int x = (int)(r % wo);
    r /= wo;
    const int y = (int)(r % ho);
    const int b = (int)(r / ho);
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        float f[8];
        unpack8(ld8(in + (((long long)b * h + 2 * y + dy) * w + 2 * x + dx) * cs_in + coff_in + c8), f);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] += f[j];
      }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] *= 0.25f;
    st8(out + (((long long)b * ho + y) * wo + x) * c + c8, pack8(acc));
  }
}

// Nearest 2x upsampling into a channel slice; h, w are the output dims;
// 8 channels per thread.
__global__ void up2_kernel(int n, int h, int w, int c, const bf16* in, bf16* out, int cs_out, int coff_out) {
  const int cv = c / 8;
  const long long total = (long long)n * h * w * cv;
  GRID_STRIDE(i, total) {
    const int c8 = (int)(i % cv) * 8;
    long long r = i / cv;
    const int x = (int)(r % w);
    r /= w;
    const int y = (int)(r % h);
    const int b = (int)(r / h);
    st8(out + (((long long)b * h + y) * w + x) * cs_out + coff_out + c8,
        ld8(in + (((long long)b * (h / 2) + y / 2) * (w / 2) + x / 2) * c + c8));
  }
}

// 8 fp32 values of an fp32 gradient (two 16-byte loads).
__device__ __forceinline__ void ld8f(const float* p, float (&f)[8]) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
  f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w; f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
}

// Gradient through the upsampling (sum of the 2x2 children of a channel
// slice of g, fp32) times [act > 0]; h, w are the fine dims; 8 channels per
// thread.
__global__ void up2_bwd_kernel(int n, int h, int w, int c, const float* g, int cs_g, int coff_g, const bf16* act,
                               bf16* out) {
  const int ho = h / 2, wo = w / 2, cv = c / 8;
  const long long total = (long long)n * ho * wo * cv;
  GRID_STRIDE(i, total) {
    const int c8 = (int)(i % cv) * 8;
    long long r = i / cv;
    const int x = (int)(r % wo);
    r /= wo;
    const int y = (int)(r % ho);
    const int b = (int)(r / ho);
    float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        float f[8];
        ld8f(g + (((long long)b * h + 2 * y + dy) * w + 2 * x + dx) * cs_g + coff_g + c8, f);
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] += f[j];
      }
    const long long o = (((long long)b * ho + y) * wo + x) * c + c8;
    float m[8];
    unpack8(ld8(act + o), m);
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = m[j] > 0.f ? a[j] : 0.f;
    st8(out + o, pack8(a));
  }
}

// Gradient at an encoder output: pooling backward (gp / 4 from the coarse
// level) plus the skip branch (a channel slice of g), times [act > 0];
// h, w are the fine dims; 8 channels per thread.
__global__ void pool2_bwd_kernel(int n, int h, int w, int c, const float* gp, const float* gs, int cs_s, int coff_s,
                                 const bf16* act, int cs_a, int coff_a, bf16* out) {
  const int cv = c / 8;
  const long long total = (long long)n * h * w * cv;
  GRID_STRIDE(i, total) {
    const int c8 = (int)(i % cv) * 8;
    long long r = i / cv;
    const int x = (int)(r % w);
    r /= w;
    const int y = (int)(r % h);
    const int b = (int)(r / h);
    const long long pix = ((long long)b * h + y) * w + x;
    float a[8], f[8], m[8];
    ld8f(gp + (((long long)b * (h / 2) + y / 2) * (w / 2) + x / 2) * c + c8, a);
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] *= 0.25f;
    if (gs != nullptr) {
      ld8f(gs + pix * cs_s + coff_s + c8, f);
#pragma unroll
      for (int j = 0; j < 8; ++j) a[j] += f[j];
    }
    unpack8(ld8(act + pix * cs_a + coff_a + c8), m);
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = m[j] > 0.f ? a[j] : 0.f;
    st8(out + pix * c + c8, pack8(a));
  }
}

// db[c] += sum over images and pixels of dy[n][c][p] (channel-major copy);
// block (split, channel).
__global__ void bias_grad_kernel(int n, long long hw, int c, const bf16* dy, float* db) {
  const int ch = blockIdx.y;
  float a = 0.f;
  const long long total = (long long)n * hw;
  GRID_STRIDE(q, total) {
    const long long b = q / hw, p = q % hw;
    a += ld(dy + (b * c + ch) * hw + p);
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(db + ch, a);
}

// fp32 [cout][cin][3][3] -> bf16 [cout][9][cin] and flipped transpose [cin][9][cout].
__global__ void pack_weights_kernel(int cout, int cin, const float* W, bf16* wt, bf16* wflip) {
  const long long total = (long long)cout * cin * 9;
  GRID_STRIDE(i, total) {
    const int t = (int)(i % 9);
    const int ci = (int)((i / 9) % cin);
    const int co = (int)(i / (9LL * cin));
    const bf16 v = st(W[i]);
    wt[((long long)co * 9 + t) * cin + ci] = v;
    if (wflip != nullptr) wflip[((long long)ci * 9 + (8 - t)) * cout + co] = v;
  }
}

__global__ void adam_kernel(long long n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd) {
  GRID_STRIDE(i, n) {
    const float gi = g[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// loss += sum (pred - target)^2 / count; grad = 2 (pred - target) / count.
__global__ void mse_kernel(long long n, const float* pred, const float* target, float inv_count, float* grad,
                           float* loss) {
  float a = 0.f;
  GRID_STRIDE(i, n) {
    const float d = pred[i] - target[i];
    grad[i] = 2.f * d * inv_count;
    a += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, a * inv_count);
}

}  // namespace

cudaError_t launch_to_chw(int n, int h, int w, int c, int cstride, int coff, const bf16* x, int copies, bf16* out,
                          cudaStream_t s) {
  const size_t smem = (size_t)(TCHW_X + 2) * c * sizeof(bf16);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(to_chw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((unsigned)((w + TCHW_X - 1) / TCHW_X), (unsigned)(n * h));
  to_chw_kernel<<<grid, 256, smem, s>>>(n, h, w, c, cstride, coff, x, copies, out);
  return cudaGetLastError();
}

cudaError_t launch_conv_in_fwd(int n, int h, int w, int c, const float* in, const float* W, const float* b, bf16* out,
                               int cstride, int coff, cudaStream_t s) {
  if (c <= 256)
    conv_in_fwd_kernel<true><<<blocks_for((long long)n * h * w), 256, (size_t)19 * c * 4, s>>>(n, h, w, c, in, W, b,
                                                                                           out, cstride, coff);
  else
    conv_in_fwd_kernel<false><<<blocks_for((long long)n * h * w), 256, 0, s>>>(n, h, w, c, in, W, b, out, cstride,
                                                                              coff);
  return cudaGetLastError();
}

cudaError_t launch_conv_in_wgrad(int n, int h, int w, int c, const float* in, const bf16* dy, int dy_cstride,
                                 float* dW, float* db, cudaStream_t s) {
  const dim3 grid(64, c);
  conv_in_wgrad_kernel<<<grid, 256, 0, s>>>(n, h, w, c, in, dy, dy_cstride, dW, db);
  return cudaGetLastError();
}

cudaError_t launch_conv_out_fwd(int n, int h, int w, int c, const bf16* in, int cstride, const float* W,
                                const float* b, float* out, cudaStream_t s) {
  if (c == 32 || c == 64) {
    const size_t smem = (size_t)3 * (COUT_TX + 2) * (c / 8) * 16 + (size_t)9 * c * 4;
    auto kern = c == 32 ? conv_out_tile_kernel<4> : conv_out_tile_kernel<8>;
    static bool set[2] = {false, false};
    if (!set[c == 64]) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      set[c == 64] = true;
    }
    const long long blocks = (long long)n * h * ((w + COUT_TX - 1) / COUT_TX);
    kern<<<(unsigned)blocks, COUT_TX, smem, s>>>(n, h, w, in, cstride, W, b, out);
    return cudaGetLastError();
  }
  conv_out_fwd_kernel<<<blocks_for((long long)n * h * w), 256, 0, s>>>(n, h, w, c, in, cstride, W, b, out);
  return cudaGetLastError();
}

cudaError_t launch_conv_out_bwd(int n, int h, int w, int c, const float* g, const float* W, const bf16* act,
                                int act_cstride, bf16* dx, float* dW, float* db, cudaStream_t s) {
  conv_out_dgrad_kernel<<<blocks_for((long long)n * h * w), 256, 0, s>>>(n, h, w, c, g, W, act, act_cstride, dx);
  const dim3 grid(64, c);
  conv_out_wgrad_kernel<<<grid, 256, 0, s>>>(n, h, w, c, g, act, act_cstride, dW, db);
  return cudaGetLastError();
}

cudaError_t launch_pool2(int n, int h, int w, int c, const bf16* in, int cs_in, int coff_in, bf16* out,
                         cudaStream_t s) {
  pool2_kernel<<<blocks_for((long long)n * (h / 2) * (w / 2) * (c / 8)), 256, 0, s>>>(n, h, w, c, in, cs_in, coff_in,
                                                                                     out);
  return cudaGetLastError();
}

cudaError_t launch_up2(int n, int h, int w, int c, const bf16* in, bf16* out, int cs_out, int coff_out,
                       cudaStream_t s) {
  up2_kernel<<<blocks_for((long long)n * h * w * (c / 8)), 256, 0, s>>>(n, h, w, c, in, out, cs_out, coff_out);
  return cudaGetLastError();
}

cudaError_t launch_up2_bwd(int n, int h, int w, int c, const float* g, int cs_g, int coff_g, const bf16* act,
                           bf16* out, cudaStream_t s) {
  up2_bwd_kernel<<<blocks_for((long long)n * (h / 2) * (w / 2) * (c / 8)), 256, 0, s>>>(n, h, w, c, g, cs_g, coff_g,
                                                                                         act, out);
  return cudaGetLastError();
}

cudaError_t launch_pool2_bwd(int n, int h, int w, int c, const float* gp, const float* gs, int cs_s, int coff_s,
                             const bf16* act, int cs_a, int coff_a, bf16* out, cudaStream_t s) {
  pool2_bwd_kernel<<<blocks_for((long long)n * h * w * (c / 8)), 256, 0, s>>>(n, h, w, c, gp, gs, cs_s, coff_s, act,
                                                                               cs_a, coff_a, out);
  return cudaGetLastError();
}

cudaError_t launch_bias_grad(int n, long long hw, int c, const bf16* dy, float* db, cudaStream_t s) {
  const dim3 grid(32, c);
  bias_grad_kernel<<<grid, 256, 0, s>>>(n, hw, c, dy, db);
  return cudaGetLastError();
}

cudaError_t launch_pack_weights(int cout, int cin, const float* W, bf16* wt, bf16* wflip, cudaStream_t s) {
  pack_weights_kernel<<<blocks_for((long long)cout * cin * 9), 256, 0, s>>>(cout, cin, W, wt, wflip);
  return cudaGetLastError();
}

cudaError_t launch_adam(long long n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2,
                        float eps, int step, float wd, cudaStream_t s) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<blocks_for(n), 256, 0, s>>>(n, p, g, m, v, lr, b1, b2, eps, c1, c2, wd);
  return cudaGetLastError();
}

cudaError_t launch_mse(long long n, const float* pred, const float* target, float* grad, float* loss,
                       cudaStream_t s) {
  mse_kernel<<<blocks_for(n), 256, 0, s>>>(n, pred, target, 1.f / (float)n, grad, loss);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace sgb
