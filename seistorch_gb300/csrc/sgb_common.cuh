// Shared device/host helpers for the seistorch_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "seistorch_gb300.h"

namespace sgb {

// Tile geometry of every stencil kernel: a CTA owns TX = 128 columns
// (32 lanes x float4) by TZ rows of one shot; NW warps split the rows.
constexpr int TX = 128;
constexpr int NW = 4;
constexpr int NTHREADS = 32 * NW;
constexpr int HX = 4;             // halo columns per side (>= radius, keeps 16-B alignment)
constexpr int SROW = TX + 2 * HX;  // floats per shared-memory row of a haloed tile
constexpr int MAX_TILE_SRC = 64;   // source points one tile may hold

// Status word written by kernels (bit flags), read once per host call.
enum : int { DEV_ERR_CAPACITY = 1 };

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int bytes) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void sts4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float comp(const float4& v, int m) {
  return m == 0 ? v.x : (m == 1 ? v.y : (m == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set_comp(float4& v, int m, float a) {
  if (m == 0) v.x = a; else if (m == 1) v.y = a; else if (m == 2) v.z = a; else v.w = a;
}

// Bytes of a 16-byte chunk starting at column x of a row of nx valid floats
// (0 outside [0, nx): zero fill == the zero padding of conv2d / roll edges).
__device__ __forceinline__ int chunk_bytes(int z, int x, int nz, int nx) {
  if (z < 0 || z >= nz || x < 0 || x >= nx) return 0;
  int n = nx - x;
  return (n >= 4 ? 4 : n) * 4;
}

// Interior box and the boundary ring saved for wavefield reconstruction.
// Ring = cells of [iz0-rt, iz1+rb) x [ix0-rl, ix1+rr) outside the box:
// top band, bottom band (full width), then left and right bands.
struct Ring {
  int iz0, iz1, ix0, ix1;
  int rt, rb, rl, rr;
  int size;  // floats per shot per step
  __host__ __device__ int width() const { return (ix1 + rr) - (ix0 - rl); }
  __host__ __device__ bool inside(int z, int x) const {
    return z >= iz0 && z < iz1 && x >= ix0 && x < ix1;
  }
  __host__ __device__ int index(int z, int x) const {
    const int W = width();
    const int xa = ix0 - rl;
    if (x < xa || x >= ix1 + rr) return -1;
    if (z >= iz0 - rt && z < iz0) return (z - (iz0 - rt)) * W + (x - xa);
    if (z >= iz1 && z < iz1 + rb) return rt * W + (z - iz1) * W + (x - xa);
    if (z >= iz0 && z < iz1) {
      const int base = (rt + rb) * W;
      const int nzi = iz1 - iz0;
      if (x < ix0) return base + (z - iz0) * rl + (x - xa);
      if (x >= ix1) return base + nzi * rl + (z - iz0) * rr + (x - ix1);
    }
    return -1;
  }
  // The cell (z, x) of slot ri in [0, size): the inverse of index().
  __host__ __device__ void cell(int ri, int& z, int& x) const {
    const int W = width();
    const int xa = ix0 - rl;
    if (ri < rt * W) {
      z = iz0 - rt + ri / W; x = xa + ri % W;
      return;
    }
    ri -= rt * W;
    if (ri < rb * W) {
      z = iz1 + ri / W; x = xa + ri % W;
      return;
    }
    ri -= rb * W;
    const int nl = (iz1 - iz0) * rl;
    if (ri < nl) {
      z = iz0 + ri / rl; x = xa + ri % rl;
      return;
    }
    ri -= nl;
    z = iz0 + ri / rr; x = ix1 + ri % rr;
  }
  // Does the tile [z0, z0+tz) x [x0, x0+tx) hold any ring cell?
  __host__ __device__ bool touches(int z0, int tz, int x0, int tx) const {
    const bool in_outer = z0 < iz1 + rb && z0 + tz > iz0 - rt && x0 < ix1 + rr && x0 + tx > ix0 - rl;
    const bool in_box = z0 >= iz0 && z0 + tz <= iz1 && x0 >= ix0 && x0 + tx <= ix1;
    return in_outer && !in_box;
  }
};

inline Ring make_ring(const sgb_grid& g, int iz0, int iz1, int ix0, int ix1, int r) {
  Ring R;
  R.iz0 = iz0; R.iz1 = iz1; R.ix0 = ix0; R.ix1 = ix1;
  R.rt = iz0 < r ? iz0 : r;
  R.rb = (g.nz - iz1) < r ? (g.nz - iz1) : r;
  R.rl = ix0 < r ? ix0 : r;
  R.rr = (g.nx - ix1) < r ? (g.nx - ix1) : r;
  const int W = R.width();
  R.size = (R.rt + R.rb) * W + (iz1 - iz0) * (R.rl + R.rr);
  return R;
}

// Second-derivative Taylor weights c_1..c_4 for orders 2..8 (the weights
// that acoustic.py:5-30 solves for), centre = -4 * sum.
struct FdWeights {
  float c[5];  // c[0] centre, c[1..4]
};
FdWeights fd_weights(int order);

int set_cuda_error(cudaError_t e);

// p[0..3] += v as one 16-byte reduction in L2 (p 16-byte aligned): the
// adjoints add every shot's gradient term into one plane with it.
__device__ __forceinline__ void red_add4(float* p, const float4& v) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
}

}  // namespace sgb

#define SGB_CUDA_CHECK(expr)                              \
  do {                                                    \
    cudaError_t _e = (expr);                              \
    if (_e != cudaSuccess) return ::sgb::set_cuda_error(_e); \
  } while (0)
