// extern "C" entry points of the learned preconditioner's tensor-core
// convolutions (kernels in nn_gemm.cu, layout kernels in nn_ops.cu).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstring>

#include "sgb_common.cuh"
#include "capi_util.cuh"
#include "nn_args.cuh"

namespace sgb {
namespace nn {
cudaError_t launch_gemm(int bn, int rb, const CUtensorMap* maps, const GemmArgs& g, dim3 grid, cudaStream_t s);
using bf16 = __nv_bfloat16;
cudaError_t launch_to_chw(int n, int h, int w, int c, int cstride, int coff, const bf16* x, int copies, bf16* out,
                          cudaStream_t s);
cudaError_t launch_conv_in_fwd(int n, int h, int w, int c, const float* in, const float* W, const float* b, bf16* out,
                               int cstride, int coff, cudaStream_t s);
cudaError_t launch_conv_in_wgrad(int n, int h, int w, int c, const float* in, const bf16* dy, int dy_cstride,
                                 float* dW, float* db, cudaStream_t s);
cudaError_t launch_conv_out_fwd(int n, int h, int w, int c, const bf16* in, int cstride, const float* W,
                                const float* b, float* out, cudaStream_t s);
cudaError_t launch_conv_out_bwd(int n, int h, int w, int c, const float* g, const float* W, const bf16* act,
                                int act_cstride, bf16* dx, float* dW, float* db, cudaStream_t s);
cudaError_t launch_pool2(int n, int h, int w, int c, const bf16* in, int cs_in, int coff_in, bf16* out,
                         cudaStream_t s);
cudaError_t launch_up2(int n, int h, int w, int c, const bf16* in, bf16* out, int cs_out, int coff_out,
                       cudaStream_t s);
cudaError_t launch_up2_bwd(int n, int h, int w, int c, const float* g, int cs_g, int coff_g, const bf16* act,
                           bf16* out, cudaStream_t s);
cudaError_t launch_pool2_bwd(int n, int h, int w, int c, const float* gp, const float* gs, int cs_s, int coff_s,
                             const bf16* act, int cs_a, int coff_a, bf16* out, cudaStream_t s);
cudaError_t launch_bias_grad(int n, long long hw, int c, const bf16* dy, float* db, cudaStream_t s);
cudaError_t launch_pack_weights(int cout, int cin, const float* W, bf16* wt, bf16* wflip, cudaStream_t s);
cudaError_t launch_adam(long long n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2,
                        float eps, int step, float wd, cudaStream_t s);
cudaError_t launch_mse(long long n, const float* pred, const float* target, float* grad, float* loss,
                       cudaStream_t s);
}  // namespace nn
}  // namespace sgb

using namespace sgb;
using namespace sgb::nn;

namespace {

using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                            const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                            CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

Encode encoder() {
  static Encode enc = nullptr;
  if (enc == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      enc = reinterpret_cast<Encode>(fn);
  }
  return enc;
}

// bf16 tiled map; dims / box innermost first, strides in bytes for dims 1..
int bf16_map(CUtensorMap* m, const void* base, int rank, const uint64_t* dims, const uint64_t* strides,
             const uint32_t* box, int row_bytes) {
  Encode enc = encoder();
  if (enc == nullptr) return -1;
  cuuint64_t gd[4], gs[3];
  cuuint32_t bx[4], es[4];
  for (int i = 0; i < rank; ++i) {
    gd[i] = dims[i];
    bx[i] = box[i];
    es[i] = 1;
  }
  for (int i = 0; i + 1 < rank; ++i) gs[i] = strides[i];
  const CUtensorMapSwizzle sw = row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), gd, gs, bx, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

bool conv_shape_ok(int n, int h, int w, int cin, int cout) {
  if (n <= 0 || h <= 0 || w <= 0 || cin <= 0 || cout <= 0) return false;
  if (cin % 32 != 0) return false;
  if (w >= 128 ? (w % 128 != 0) : (w < 64 || 128 % w != 0)) return false;
  return true;
}

int pick_bn(int c) { return c >= 128 ? 128 : (c > 32 ? 64 : 32); }

}  // namespace

extern "C" {

int sgb_nn_conv3x3(const sgb_nn_conv* c, sgb_stream_t stream) {
  if (c == nullptr || c->x == nullptr || c->wt == nullptr) return SGB_ERR_ARG;
  if (c->out_bf16 == nullptr && c->out_f32 == nullptr) return SGB_ERR_ARG;
  if (!conv_shape_ok(c->n, c->h, c->w, c->cin, c->cout)) return SGB_ERR_SHAPE;
  if (c->out_cstride < c->out_coff + c->cout || (c->mask != nullptr && c->mask_cstride < c->cout))
    return SGB_ERR_SHAPE;
  if (!aligned16(c->x) || !aligned16(c->wt)) return SGB_ERR_ALIGN;
  const int rb = c->cin % 64 == 0 ? 128 : 64;
  const int bn = pick_bn(c->cout);
  GemmArgs g;
  std::memset(&g, 0, sizeof(g));
  g.mode = MODE_CONV;
  g.N = c->n;
  g.H = c->h;
  g.W = c->w;
  g.Cin = c->cin;
  g.Cout = c->cout;
  g.TW = c->w < 128 ? c->w : 128;
  g.TH = 128 / g.TW;
  g.tiles_x = c->w / g.TW;
  g.tiles_y = (c->h + g.TH - 1) / g.TH;
  g.nchunk = c->cin / (rb / 2);
  g.kiters = 9 * g.nchunk;
  g.bias = c->bias;
  g.relu = c->relu;
  g.mask = static_cast<const __nv_bfloat16*>(c->mask);
  g.mask_cstride = c->mask_cstride;
  g.out_bf16 = static_cast<__nv_bfloat16*>(c->out_bf16);
  g.out_f32 = c->out_f32;
  g.out_cstride = c->out_cstride;
  g.out_coff = c->out_coff;
  g.status = status_ptr();
  CUtensorMap maps[4];
  const uint64_t eb = 2;
  {
    const uint64_t dims[4] = {(uint64_t)c->cin, (uint64_t)c->w, (uint64_t)c->h, (uint64_t)c->n};
    const uint64_t st[3] = {c->cin * eb, (uint64_t)c->w * c->cin * eb, (uint64_t)c->h * c->w * c->cin * eb};
    const uint32_t box[4] = {(uint32_t)(rb / 2), (uint32_t)g.TW, (uint32_t)g.TH, 1};
    if (bf16_map(&maps[0], c->x, 4, dims, st, box, rb)) return SGB_ERR_CUDA;
  }
  {
    const uint64_t dims[3] = {(uint64_t)c->cin, 9, (uint64_t)c->cout};
    const uint64_t st[2] = {c->cin * eb, 9ull * c->cin * eb};
    const uint32_t box[3] = {(uint32_t)(rb / 2), 1, (uint32_t)bn};
    if (bf16_map(&maps[1], c->wt, 3, dims, st, box, rb)) return SGB_ERR_CUDA;
  }
  maps[2] = maps[1];
  maps[3] = maps[1];
  const dim3 grid((unsigned)(c->n * g.tiles_x * g.tiles_y), (unsigned)((c->cout + bn - 1) / bn), 1);
  SGB_CUDA_CHECK(launch_gemm(bn, rb, maps, g, grid, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_conv3x3_wgrad(const sgb_nn_wgrad* p, sgb_stream_t stream) {
  if (p == nullptr || p->dy_chw == nullptr || p->dw == nullptr) return SGB_ERR_ARG;
  for (int k = 0; k < 3; ++k)
    if (p->x_chw[k] == nullptr) return SGB_ERR_ARG;
  if (p->n <= 0 || p->h <= 0 || p->cin <= 0 || p->cout <= 0 || p->w <= 0 || p->w % 64 != 0) return SGB_ERR_SHAPE;
  if (p->cin % 8 != 0 || p->cout % 8 != 0) return SGB_ERR_SHAPE;
  if (!aligned16(p->dy_chw) || !aligned16(p->x_chw[0]) || !aligned16(p->x_chw[1]) || !aligned16(p->x_chw[2]))
    return SGB_ERR_ALIGN;
  const int bn = pick_bn(p->cin);
  GemmArgs g;
  std::memset(&g, 0, sizeof(g));
  g.mode = MODE_WGRAD;
  g.N = p->n;
  g.H = p->h;
  g.W = p->w;
  g.Cin = p->cin;
  g.Cout = p->cout;
  g.wchunks = p->w / 64;
  g.kiters = p->n * p->h * g.wchunks;
  int splits = (g.kiters + 127) / 128;
  if (splits > 64) splits = 64;
  g.k_per_split = (g.kiters + splits - 1) / splits;
  splits = (g.kiters + g.k_per_split - 1) / g.k_per_split;
  g.out_f32 = p->dw;
  g.status = status_ptr();
  CUtensorMap maps[4];
  const uint64_t eb = 2;
  {
    const uint64_t dims[4] = {(uint64_t)p->w, (uint64_t)p->h, (uint64_t)p->cout, (uint64_t)p->n};
    const uint64_t st[3] = {p->w * eb, (uint64_t)p->h * p->w * eb, (uint64_t)p->cout * p->h * p->w * eb};
    const uint32_t box[4] = {64, 1, 128, 1};
    if (bf16_map(&maps[0], p->dy_chw, 4, dims, st, box, 128)) return SGB_ERR_CUDA;
  }
  for (int k = 0; k < 3; ++k) {
    const uint64_t dims[4] = {(uint64_t)p->w, (uint64_t)p->h, (uint64_t)p->cin, (uint64_t)p->n};
    const uint64_t st[3] = {p->w * eb, (uint64_t)p->h * p->w * eb, (uint64_t)p->cin * p->h * p->w * eb};
    const uint32_t box[4] = {64, 1, (uint32_t)bn, 1};
    if (bf16_map(&maps[1 + k], p->x_chw[k], 4, dims, st, box, 128)) return SGB_ERR_CUDA;
  }
  const int mtiles = (p->cout + 127) / 128;
  const dim3 grid((unsigned)splits, (unsigned)((p->cin + bn - 1) / bn), (unsigned)(9 * mtiles));
  SGB_CUDA_CHECK(launch_gemm(bn, 128, maps, g, grid, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_to_chw(int32_t n, int32_t h, int32_t w, int32_t c, int32_t cstride, int32_t coff, const void* x_nhwc,
                  int32_t copies, void* out, sgb_stream_t stream) {
  if (x_nhwc == nullptr || out == nullptr || (copies != 1 && copies != 3)) return SGB_ERR_ARG;
  if (n <= 0 || h <= 0 || w <= 0 || c <= 0 || cstride < coff + c || coff < 0) return SGB_ERR_SHAPE;
  if (c % 8 || cstride % 8 || coff % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_to_chw(n, h, w, c, cstride, coff, static_cast<const bf16*>(x_nhwc), copies,
                               static_cast<bf16*>(out), (cudaStream_t)stream));
  return SGB_OK;
}

#define NN_DIMS_OK(n, h, w, c) ((n) > 0 && (h) > 0 && (w) > 0 && (c) > 0)
#define BF(p) static_cast<const bf16*>(p)
#define BFW(p) static_cast<bf16*>(p)

int sgb_nn_conv_in(int32_t n, int32_t h, int32_t w, int32_t c, const float* in, const float* W, const float* b,
                   void* out, int32_t cstride, int32_t coff, sgb_stream_t stream) {
  if (in == nullptr || W == nullptr || b == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || cstride < coff + c || coff < 0) return SGB_ERR_SHAPE;
  if (c % 8 || cstride % 8 || coff % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_conv_in_fwd(n, h, w, c, in, W, b, BFW(out), cstride, coff, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_conv_in_wgrad(int32_t n, int32_t h, int32_t w, int32_t c, const float* in, const void* dy,
                         int32_t dy_cstride, float* dW, float* db, sgb_stream_t stream) {
  if (in == nullptr || dy == nullptr || dW == nullptr || db == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || dy_cstride < c) return SGB_ERR_SHAPE;
  SGB_CUDA_CHECK(launch_conv_in_wgrad(n, h, w, c, in, BF(dy), dy_cstride, dW, db, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_conv_out(int32_t n, int32_t h, int32_t w, int32_t c, const void* in, int32_t cstride, const float* W,
                    const float* b, float* out, sgb_stream_t stream) {
  if (in == nullptr || W == nullptr || b == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || cstride < c) return SGB_ERR_SHAPE;
  if (c % 8 || cstride % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_conv_out_fwd(n, h, w, c, BF(in), cstride, W, b, out, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_conv_out_bwd(int32_t n, int32_t h, int32_t w, int32_t c, const float* g, const float* W, const void* act,
                        int32_t act_cstride, void* dx, float* dW, float* db, sgb_stream_t stream) {
  if (g == nullptr || W == nullptr || act == nullptr || dx == nullptr || dW == nullptr || db == nullptr)
    return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || act_cstride < c) return SGB_ERR_SHAPE;
  if (c % 8 || act_cstride % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_conv_out_bwd(n, h, w, c, g, W, BF(act), act_cstride, BFW(dx), dW, db, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_pool2(int32_t n, int32_t h, int32_t w, int32_t c, const void* in, int32_t cs_in, int32_t coff_in,
                 void* out, sgb_stream_t stream) {
  if (in == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || h % 2 || w % 2 || cs_in < coff_in + c || coff_in < 0) return SGB_ERR_SHAPE;
  if (c % 8 || cs_in % 8 || coff_in % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_pool2(n, h, w, c, BF(in), cs_in, coff_in, BFW(out), (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_up2(int32_t n, int32_t h, int32_t w, int32_t c, const void* in, void* out, int32_t cs_out,
               int32_t coff_out, sgb_stream_t stream) {
  if (in == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || h % 2 || w % 2 || cs_out < coff_out + c || coff_out < 0) return SGB_ERR_SHAPE;
  if (c % 8 || cs_out % 8 || coff_out % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_up2(n, h, w, c, BF(in), BFW(out), cs_out, coff_out, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_up2_bwd(int32_t n, int32_t h, int32_t w, int32_t c, const float* g, int32_t cs_g, int32_t coff_g,
                   const void* act, void* out, sgb_stream_t stream) {
  if (g == nullptr || act == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || h % 2 || w % 2 || cs_g < coff_g + c || coff_g < 0) return SGB_ERR_SHAPE;
  if (c % 8 || cs_g % 8 || coff_g % 8) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_up2_bwd(n, h, w, c, g, cs_g, coff_g, BF(act), BFW(out), (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_pool2_bwd(int32_t n, int32_t h, int32_t w, int32_t c, const float* gp, const float* gs, int32_t cs_s,
                     int32_t coff_s, const void* act, int32_t cs_a, int32_t coff_a, void* out, sgb_stream_t stream) {
  if (gp == nullptr || act == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (!NN_DIMS_OK(n, h, w, c) || h % 2 || w % 2 || cs_a < coff_a + c || (gs != nullptr && cs_s < coff_s + c))
    return SGB_ERR_SHAPE;
  if (c % 8 || cs_a % 8 || coff_a % 8 || (gs != nullptr && (cs_s % 8 || coff_s % 8))) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_pool2_bwd(n, h, w, c, gp, gs, cs_s, coff_s, BF(act), cs_a, coff_a, BFW(out),
                                  (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_bias_grad(int32_t n, int64_t hw, int32_t c, const void* dy_chw, float* db, sgb_stream_t stream) {
  if (dy_chw == nullptr || db == nullptr) return SGB_ERR_ARG;
  if (n <= 0 || hw <= 0 || c <= 0) return SGB_ERR_SHAPE;
  SGB_CUDA_CHECK(launch_bias_grad(n, hw, c, BF(dy_chw), db, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_pack_weights(int32_t cout, int32_t cin, const float* W, void* wt, void* wflip, sgb_stream_t stream) {
  if (W == nullptr || wt == nullptr) return SGB_ERR_ARG;
  if (cout <= 0 || cin <= 0) return SGB_ERR_SHAPE;
  SGB_CUDA_CHECK(launch_pack_weights(cout, cin, W, BFW(wt), BFW(wflip), (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_adam(int64_t n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                int32_t step, float wd, sgb_stream_t stream) {
  if (p == nullptr || g == nullptr || m == nullptr || v == nullptr) return SGB_ERR_ARG;
  if (n <= 0 || step < 1) return SGB_ERR_ARG;
  SGB_CUDA_CHECK(launch_adam(n, p, g, m, v, lr, b1, b2, eps, step, wd, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_nn_mse(int64_t n, const float* pred, const float* target, float* grad, float* loss, sgb_stream_t stream) {
  if (pred == nullptr || target == nullptr || grad == nullptr || loss == nullptr) return SGB_ERR_ARG;
  if (n <= 0) return SGB_ERR_SHAPE;
  SGB_CUDA_CHECK(launch_mse(n, pred, target, grad, loss, (cudaStream_t)stream));
  return SGB_OK;
}

}  // extern "C"
