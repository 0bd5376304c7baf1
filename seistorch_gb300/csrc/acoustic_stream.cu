// Host side of the streaming kernels: TMA tensor maps and the variant
// selection shared by acoustic_stream_fwd.cu and acoustic_stream_bwd.cu.
#include "stream_common.cuh"

namespace sgb {


static cuuint32_t u32(uint32_t v) { return static_cast<cuuint32_t>(v); }

int make_tmap_f32(CUtensorMap* map, const float* base, int rank, const uint64_t* dims,
                  const uint64_t* strides_bytes, const uint32_t* box) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  if (encode == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || fn == nullptr)
      return -1;
    encode = reinterpret_cast<Encode>(fn);
  }
  cuuint64_t gd[3], gs[2];
  cuuint32_t bx[3], es[3];
  for (int i = 0; i < rank; ++i) {
    gd[i] = dims[i];
    bx[i] = u32(box[i]);
    es[i] = 1;
  }
  for (int i = 0; i + 1 < rank; ++i) gs[i] = strides_bytes[i];
  CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, const_cast<float*>(base), gd, gs, bx,
                      es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

// Tensor maps of a [nshots][nz][pitch] field with a box of boxw columns,
// rb rows and bs shots.
int field_map(CUtensorMap* m, const float* p, int nz, int nx, int pitch, int nshots, int boxw, int rb, int bs) {
  const uint64_t dims[3] = {(uint64_t)nx, (uint64_t)nz, (uint64_t)nshots};
  const uint64_t st[2] = {(uint64_t)pitch * 4, (uint64_t)nz * pitch * 4};
  const uint32_t box[3] = {(uint32_t)boxw, (uint32_t)rb, (uint32_t)bs};
  return make_tmap_f32(m, p, 3, dims, st, box);
}
int coef_map(CUtensorMap* m, const float* coef, int nz, int nx, int pitch, int rb) {
  const uint64_t dims[3] = {(uint64_t)nx, (uint64_t)nz, 2};
  const uint64_t st[2] = {(uint64_t)pitch * 4, (uint64_t)nz * pitch * 4};
  const uint32_t box[3] = {(uint32_t)TX, (uint32_t)rb, 2};
  return make_tmap_f32(m, coef, 3, dims, st, box);
}
int plane_map(CUtensorMap* m, const float* p, int nz, int nx, int pitch, int boxw, int rb) {
  const uint64_t dims[2] = {(uint64_t)nx, (uint64_t)nz};
  const uint64_t st[1] = {(uint64_t)pitch * 4};
  const uint32_t box[2] = {(uint32_t)boxw, (uint32_t)rb};
  return make_tmap_f32(m, p, 2, dims, st, box);
}

// Variant selection: fwd_cfg / bwd_cfg index the (rows per tile, warps per
// CTA) tables of acoustic_stream_fwd.cu / acoustic_stream_bwd.cu, habc_cfg
// the variants of the second-order HABC forward.
int g_fwd_cfg = 4, g_bwd_cfg = 4, g_habc_fwd_cfg = 0;
constexpr int N_FWD = 6, N_BWD = 6, N_HABC_FWD = 6;

int set_stream_config(int fwd, int bwd, int habc) {
  if (fwd < 0 || fwd >= N_FWD || bwd < 0 || bwd >= N_BWD || habc < 0 || habc >= N_HABC_FWD) return -1;
  g_fwd_cfg = fwd;
  g_bwd_cfg = bwd;
  g_habc_fwd_cfg = habc;
  return 0;
}

}  // namespace sgb
