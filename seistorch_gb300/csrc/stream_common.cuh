// Shared pieces of the TMA tile-pipeline acoustic PML kernels (forward step
// in acoustic_stream_fwd.cu, fused boundary-saving adjoint step in
// acoustic_stream_bwd.cu).
//
// A persistent CTA walks tiles t = blockIdx.x + k * gridDim.x (shot fastest,
// then 128-column strip, then TZ-row band).  The haloed stencil rows of a
// tile -- (TZ + 2R) x W floats, W = 136 or 144 (see Row<R>) -- arrive in one
// of S shared-memory stages by TMA (cp.async.bulk.tensor); out-of-bounds box
// elements read as zero, which is the zero padding of conv2d(padding=order/2)
// (acoustic.py:71).  Thread 0 re-arms a stage with tile k+S as soon as all
// warps are done with tile k.  The point operands (previous field,
// coefficient planes) are fetched with 16-byte global loads issued before the
// stage wait, so their latency overlaps it; the coefficient planes are shared
// by all shots and stay in L2.  Each warp computes TZ/NW rows with a fully
// unrolled register window along z; lanes own 4 adjacent columns (float4),
// x-neighbours come from the staged row.  Every mbarrier wait is bounded and
// a timeout ends the CTA's loop at the next barrier.
#pragma once
#include <algorithm>

#include "sgb_common.cuh"
#include "acoustic_args.cuh"
#include "tma.cuh"

namespace sgb {

constexpr unsigned FULL = 0xffffffffu;

constexpr int round32(int n) { return (n + 31) / 32 * 32; }

// Width W of a staged stencil row and the offset LO of column x0 in it: the
// box spans columns [x0 - LO, x0 - LO + W).  136 floats (LO = 4) for even
// radii, 144 (LO = 8) for odd radii (keeps 2R rows a multiple of 128 bytes).
template <int R>
struct Row {
  static constexpr int W = (R % 2 == 0) ? TX + 8 : TX + 16;
  static constexpr int LO = (W - TX) / 2;
};

// Tile t -> (shot, strip, band); 32-bit arithmetic.
struct Tile {
  int b, x0, z0;
};
__device__ __forceinline__ Tile tile_geom(int t, int nshots, int ntx, int tz) {
  Tile g;
  g.b = t % nshots;
  const int rest = t / nshots;
  g.x0 = (rest % ntx) * TX;
  g.z0 = (rest / ntx) * tz;
  return g;
}

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// Value of component (rx & 3) of lane (rx >> 2)'s float4, for every lane.
__device__ __forceinline__ float gather_lane(const float4& v, int rx) {
  const int src = rx >> 2, m = rx & 3;
  const float a = __shfl_sync(FULL, v.x, src), b = __shfl_sync(FULL, v.y, src);
  const float c = __shfl_sync(FULL, v.z, src), d = __shfl_sync(FULL, v.w, src);
  return m == 0 ? a : (m == 1 ? b : (m == 2 ? c : d));
}

// Cross-stencil Laplacian (without 1/h^2) of the 4 columns of a lane at the
// centre row of `win`, x-neighbours from the staged row `srow` (its element
// Row<R>::LO is column x0).
template <int R>
__device__ __forceinline__ float4 lap_row(const float4 (&win)[2 * R + 1], const float* srow, int lane,
                                          const FdWeights& w) {
  const float4 l = lds4(srow + Row<R>::LO - 4 + 4 * lane);
  const float4 r = lds4(srow + Row<R>::LO + 4 + 4 * lane);
  const float4 c = win[R];
  const float a[12] = {l.x, l.y, l.z, l.w, c.x, c.y, c.z, c.w, r.x, r.y, r.z, r.w};
  float4 L;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    float s = w.c[0] * a[4 + m];
#pragma unroll
    for (int j = 1; j <= R; ++j)
      s = fmaf(w.c[j], (a[4 + m + j] + a[4 + m - j]) + (comp(win[R + j], m) + comp(win[R - j], m)), s);
    set_comp(L, m, s);
  }
  return L;
}

// Sources of shot b in rows [zlo, zlo + nrow) and columns [x0, x0 + 128):
// one candidate per lane (the first 32 sources of the shot), as a ballot mask
// plus (row offset, column offset, value) in the owning lane.
struct WarpSrc {
  unsigned mask;
  int zl, xl;
  float v;
};
__device__ __forceinline__ WarpSrc warp_sources(int lane, int b, int zlo, int nrow, int x0, const int* src_ptr,
                                                const int* src_z, const int* src_x, const int* src_wrow,
                                                const float* wavelet, int nt, int t, int* status) {
  WarpSrc s{0u, -1, 0, 0.f};
  const int p0 = src_ptr[b], p1 = src_ptr[b + 1];
  const int q = p0 + lane;
  if (q < p1) {
    const int zs = src_z[q] - zlo, xs = src_x[q] - x0;
    if (zs >= 0 && zs < nrow && xs >= 0 && xs < TX) {
      s.zl = zs;
      s.xl = xs;
      s.v = wavelet[(long long)src_wrow[q] * nt + t];
    }
  }
  s.mask = __ballot_sync(FULL, s.zl >= 0);
  if (p1 - p0 > 32 && lane == 0) atomicOr(status, DEV_ERR_CAPACITY);
  return s;
}

// Add (sign = +1) or subtract (-1) the sources of local row i to v.
__device__ __forceinline__ void apply_sources(const WarpSrc& s, int i, int lane, float sign, float4& v) {
  unsigned m = s.mask;
  while (m) {
    const int srcl = __ffs(m) - 1;
    m &= m - 1;
    const int zl = __shfl_sync(FULL, s.zl, srcl), xl = __shfl_sync(FULL, s.xl, srcl);
    const float val = __shfl_sync(FULL, s.v, srcl);
    if (zl == i && (xl >> 2) == lane) set_comp(v, xl & 3, comp(v, xl & 3) + sign * val);
  }
}

// This CTA's share of a boundary-ring copy between a field
// [nshots][nz][pitch] and its slots [nshots][ring.size] (slot order of
// Ring::index): scatter = slots -> field, else field -> slots.  Four
// elements per thread and round: their loads are issued together.
__device__ __forceinline__ void ring_copy_share(const Ring& ring, int nshots, int pitch, long long sstride,
                                                float* field, float* slots, bool scatter) {
  const long long n = (long long)nshots * ring.size;
  const long long stride = (long long)gridDim.x * blockDim.x;
  auto cell_ptr = [&](long long i) -> float* {
    const int b = (int)(i / ring.size);
    int z, x;
    ring.cell((int)(i - (long long)b * ring.size), z, x);
    return field + b * sstride + (long long)z * pitch + x;
  };
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    float* f[4];
    float v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) f[q] = cell_ptr(i + q * stride);
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = scatter ? slots[i + q * stride] : *f[q];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (scatter)
        *f[q] = v[q];
      else
        slots[i + q * stride] = v[q];
    }
  }
  for (; i < n; i += stride) {
    float* f = cell_ptr(i);
    if (scatter)
      *f = slots[i];
    else
      slots[i] = *f;
  }
}

template <class Kern>
static int resident_blocks(Kern kern, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem) != cudaSuccess || nb < 1) nb = 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return nb * (sms > 0 ? sms : 152);
}

// Variant selection shared with the host (acoustic_stream.cu).
extern int g_fwd_cfg, g_bwd_cfg, g_habc_fwd_cfg;

}  // namespace sgb
