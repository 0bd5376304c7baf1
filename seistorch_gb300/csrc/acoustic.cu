// 2nd-order-in-time acoustic kernels (PML and HABC) for sm_103a.
//
// Stencil: L(u) = c0 u + sum_j c_j (u[z+j] + u[z-j] + u[x+j] + u[x-j]) with
// zero padding (conv2d(padding=order/2), seistorch/equations2d/acoustic.py:60-71).
// Update: u+ = g (u - u-) + u- + k L(u)  (algebraically acoustic.py:81-84 with
// g = 2/(1+d dt), k = vp^2 dt^2/(h^2 (1+d dt))).
//
// Tiling: one CTA = 128 columns x TZ rows of one shot.  The haloed u tile and
// the point tiles (u-, g, k) are staged into shared memory with 16-byte
// cp.async copies (zero-filled outside the grid), all issued before any
// compute so every load of the tile is in flight at once; each thread then
// owns 4 adjacent columns (float4) and streams its warp's rows keeping the
// z-window of the stencil in registers, reading x-neighbours from the
// shared row.
#include <algorithm>

#include "sgb_common.cuh"
#include "acoustic_args.cuh"
#include "habc_blend.cuh"

namespace sgb {

// ------------------------------------------------------------ forward ---


template <int TZ, int HR>
struct FwdTile {
  const float* s_u;
  const float* s_um;
  int z0, x0;
  long long base;
  int pitch;
  const float* __restrict__ u;
  const float* __restrict__ um;
  __device__ __forceinline__ float U(int z, int x) const {
    const int r = z - (z0 - HR), c = x - (x0 - HX);
    if (r >= 0 && r < TZ + 2 * HR && c >= 0 && c < SROW) return s_u[r * SROW + c];
    return u[base + (long long)z * pitch + x];
  }
  __device__ __forceinline__ float P(int z, int x) const {
    const int r = z - z0, c = x - x0;
    if (r >= 0 && r < TZ && c >= 0 && c < TX) return s_um[r * TX + c];
    return um[base + (long long)z * pitch + x];
  }
};

template <int R>
__device__ __forceinline__ float4 lap4(const float4 (&win)[2 * R + 1], const float4& left,
                                       const float4& right, const FdWeights& w) {
  const float a[12] = {left.x, left.y, left.z, left.w, win[R].x, win[R].y, win[R].z, win[R].w,
                       right.x, right.y, right.z, right.w};
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

// The x and z parts of lap4 (1-D second differences, centre -2 sum c).
template <int R>
__device__ __forceinline__ void lap4_xz(const float4 (&win)[2 * R + 1], const float4& left, const float4& right,
                                        const FdWeights& w, float4& Lx, float4& Lz) {
  const float a[12] = {left.x, left.y, left.z, left.w, win[R].x, win[R].y, win[R].z, win[R].w,
                       right.x, right.y, right.z, right.w};
  const float c0 = 0.5f * w.c[0];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    float sx = c0 * a[4 + m], sz = c0 * a[4 + m];
#pragma unroll
    for (int j = 1; j <= R; ++j) {
      sx = fmaf(w.c[j], a[4 + m + j] + a[4 + m - j], sx);
      sz = fmaf(w.c[j], comp(win[R + j], m) + comp(win[R - j], m), sz);
    }
    set_comp(Lx, m, sx);
    set_comp(Lz, m, sz);
  }
}

template <int R, int TZ, bool HABC>
__global__ void __launch_bounds__(NTHREADS) acoustic_fwd_kernel(const AcStepArgs a) {
  constexpr int HR = (HABC && R < 2) ? 2 : R;
  constexpr int RPW = TZ / NW;
  extern __shared__ __align__(16) float smem[];
  float* s_u = smem;                           // (TZ + 2HR) x SROW
  float* s_um = s_u + (TZ + 2 * HR) * SROW;     // TZ x TX
  int* s_src = reinterpret_cast<int*>(s_um + TZ * TX);  // [2 * MAX_TILE_SRC] + count
  float* s_srcv = reinterpret_cast<float*>(s_src + 2 * MAX_TILE_SRC + 1);

  const int tid = threadIdx.x;
  const int b = blockIdx.x % a.nshots;
  const int tile = blockIdx.x / a.nshots;
  const int x0 = (tile % a.ntx) * TX;
  const int z0 = (tile / a.ntx) * TZ;
  const long long base = (long long)b * a.sstride;

  // ---- stage the tile: every 16-byte chunk in flight before any compute
  constexpr int UCH = SROW / 4;
  for (int c = tid; c < (TZ + 2 * HR) * UCH; c += NTHREADS) {
    const int r = c / UCH, cc = c - r * UCH;
    const int z = z0 - HR + r, x = x0 - HX + 4 * cc;
    const int nb = chunk_bytes(z, x, a.nz, a.nx);
    cp_async16(s_u + r * SROW + 4 * cc, nb ? a.u + base + (long long)z * a.pitch + x : a.u, nb);
  }
  constexpr int PCH = TX / 4;
  for (int c = tid; c < TZ * PCH; c += NTHREADS) {
    const int r = c / PCH, cc = c - r * PCH;
    const int z = z0 + r, x = x0 + 4 * cc;
    const int nb = chunk_bytes(z, x, a.nz, a.nx);
    const long long off = (long long)z * a.pitch + x;
    cp_async16(s_um + r * TX + 4 * cc, nb ? a.um + base + off : a.um, nb);
  }
  cp_async_commit();
  // sources of this shot that fall in the tile
  if (tid == 0) s_src[2 * MAX_TILE_SRC] = 0;
  __syncthreads();
  if (a.src_ptr != nullptr) {
    const int p0 = a.src_ptr[b], p1 = a.src_ptr[b + 1];
    for (int q = p0 + tid; q < p1; q += NTHREADS) {
      const int zs = a.src_z[q] - z0, xs = a.src_x[q] - x0;
      if (zs >= 0 && zs < TZ && xs >= 0 && xs < TX) {
        const int slot = atomicAdd(&s_src[2 * MAX_TILE_SRC], 1);
        if (slot < MAX_TILE_SRC) {
          s_src[2 * slot] = zs;
          s_src[2 * slot + 1] = xs;
          s_srcv[slot] = a.wavelet[(long long)a.src_wrow[q] * a.nt + a.t];
        } else {
          atomicOr(a.status, DEV_ERR_CAPACITY);
        }
      }
    }
  }
  cp_async_wait_all();
  __syncthreads();
  const int nsrc = min(s_src[2 * MAX_TILE_SRC], MAX_TILE_SRC);

  const int lane = tid & 31, wid = tid >> 5;
  const int xl = 4 * lane;
  const int x = x0 + xl;
  const int sr0 = HR + wid * RPW;  // shared row of this warp's first output row
  FwdTile<TZ, HR> T{s_u, s_um, z0, x0, base, a.pitch, a.u, a.um};

  float4 win[2 * R + 1];
#pragma unroll
  for (int j = 0; j < 2 * R; ++j) win[j] = lds4(s_u + (sr0 - R + j) * SROW + HX + xl);
#pragma unroll
  for (int i = 0; i < RPW; ++i) {
    const int sr = sr0 + i;
    const int lr = wid * RPW + i;  // local output row
    const int z = z0 + lr;
    win[2 * R] = lds4(s_u + (sr + R) * SROW + HX + xl);
    const float4 left = lds4(s_u + sr * SROW + xl);
    const float4 right = lds4(s_u + sr * SROW + 2 * HX + xl);
    const float4 L = lap4<R>(win, left, right, a.w);
    const float4 vm = lds4(s_um + lr * TX + xl);
    // coefficient rows straight from L2 (shared by every shot's tile; each
    // cell reads only its own value, so they need no staging)
    const bool cin = z < a.nz && x < a.nx;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 vg = cin ? __ldg(reinterpret_cast<const float4*>(a.g + (long long)z * a.pitch + x)) : zero4;
    const float4 vk = cin ? __ldg(reinterpret_cast<const float4*>(a.k + (long long)z * a.pitch + x)) : zero4;
    float4 y;
    if (HABC && R == 1 && a.rho_c != nullptr) {  // variable density: C D(u)
      const long long po = (long long)z * a.pitch + x, pl = (long long)a.nz * a.pitch;
      auto ld = [&](int q) {
        return cin ? __ldg(reinterpret_cast<const float4*>(a.rho_c + q * pl + po)) : zero4;
      };
      const float4 C4 = ld(0), bxp = ld(1), bxn = ld(2), bzp = ld(3), bzn = ld(4);
      const float xs[6] = {left.w, win[R].x, win[R].y, win[R].z, win[R].w, right.x};
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float c = xs[m + 1];
        const float D = comp(bxp, m) * (xs[m + 2] - c) - comp(bxn, m) * (c - xs[m]) +
                        comp(bzp, m) * (comp(win[R + 1], m) - c) - comp(bzn, m) * (c - comp(win[R - 1], m));
        set_comp(y, m, fmaf(comp(C4, m), D, fmaf(comp(vg, m), c - comp(vm, m), comp(vm, m))));
      }
    } else if (HABC && a.kz != nullptr) {  // VTI: k Lx + kz Lz
      float4 Lx, Lz;
      lap4_xz<R>(win, left, right, a.w, Lx, Lz);
      const float4 vz = cin ? __ldg(reinterpret_cast<const float4*>(a.kz + (long long)z * a.pitch + x)) : zero4;
      y.x = fmaf(vk.x, Lx.x, fmaf(vz.x, Lz.x, fmaf(vg.x, win[R].x - vm.x, vm.x)));
      y.y = fmaf(vk.y, Lx.y, fmaf(vz.y, Lz.y, fmaf(vg.y, win[R].y - vm.y, vm.y)));
      y.z = fmaf(vk.z, Lx.z, fmaf(vz.z, Lz.z, fmaf(vg.z, win[R].z - vm.z, vm.z)));
      y.w = fmaf(vk.w, Lx.w, fmaf(vz.w, Lz.w, fmaf(vg.w, win[R].w - vm.w, vm.w)));
    } else {
      y.x = fmaf(vk.x, L.x, fmaf(vg.x, win[R].x - vm.x, vm.x));
      y.y = fmaf(vk.y, L.y, fmaf(vg.y, win[R].y - vm.y, vm.y));
      y.z = fmaf(vk.z, L.z, fmaf(vg.z, win[R].z - vm.z, vm.z));
      y.w = fmaf(vk.w, L.w, fmaf(vg.w, win[R].w - vm.w, vm.w));
    }
    if (z < a.nz && x < a.nx) {
      const long long po = (long long)z * a.pitch + x;
      if (a.born_out != nullptr) {  // m k L(u): the scattered field's source
        const float4 mm = *reinterpret_cast<const float4*>(a.born_m + po);
        *reinterpret_cast<float4*>(a.born_out + base + po) =
            make_float4(mm.x * (vk.x * L.x), mm.y * (vk.y * L.y), mm.z * (vk.z * L.z), mm.w * (vk.w * L.w));
      }
      if (a.born_in != nullptr) {
        const float4 sb = *reinterpret_cast<const float4*>(a.born_in + base + po);
        y = make_float4(y.x + sb.x, y.y + sb.y, y.z + sb.z, y.w + sb.w);
      }
      // the blend only on strip cells; one copy of its code (not unrolled),
      // so the row loop stays small in the instruction cache
      const bool strip_lane = z < a.hw || z >= a.nz - a.hw || x < a.hw || x + 3 >= a.nx - a.hw;
      if (HABC && strip_lane) {
#pragma unroll 1
        for (int m = 0; m < 4; ++m)
          if (x + m < a.nx) set_comp(y, m, habc_point(T, a, z, x + m, comp(y, m)));
      }
      for (int s = 0; s < nsrc; ++s) {
        if (s_src[2 * s] == lr && (s_src[2 * s + 1] >> 2) == lane) {
          const int m = s_src[2 * s + 1] & 3;
          set_comp(y, m, comp(y, m) + s_srcv[s]);
        }
      }
      *reinterpret_cast<float4*>(a.un + base + (long long)z * a.pitch + x) = y;
      if (a.illum != nullptr) {
#pragma unroll
        for (int m = 0; m < 4; ++m)
          if (x + m < a.nx) atomicAdd(a.illum + (long long)z * a.pitch + x + m, comp(y, m) * comp(y, m));
      }
    }
#pragma unroll
    for (int j = 0; j < 2 * R; ++j) win[j] = win[j + 1];
  }

  // ---- receivers: read back the finished tile (same-CTA writes are visible)
  if (a.records != nullptr) {
    __syncthreads();
    for (int lr = wid; lr < TZ; lr += NW) {
      const int z = z0 + lr;
      if (z >= a.nz) break;
      const int p0 = a.rec_row_ptr[b * a.nz + z], p1 = a.rec_row_ptr[b * a.nz + z + 1];
      for (int q = p0 + lane; q < p1; q += 32) {
        const int rx = a.rec_x[q];
        if (rx >= x0 && rx < x0 + TX)
          a.records[(long long)a.rec_col[q] * a.nch] = a.un[base + (long long)z * a.pitch + rx];
      }
    }
  }
}

// ------------------------------------------- single-step VJP (PML) ---


template <int R, int TZ>
__global__ void __launch_bounds__(NTHREADS) acoustic_vjp_kernel(const AcVjpArgs a) {
  constexpr int HR = R;
  constexpr int RPW = TZ / NW;
  extern __shared__ __align__(16) float smem[];
  float* s_u = smem;
  float* s_y = s_u + (TZ + 2 * HR) * SROW;  // gy, then k*gy
  float* s_k = s_y + (TZ + 2 * HR) * SROW;
  const int tid = threadIdx.x;
  const int b = blockIdx.x % a.nshots;
  const int tile = blockIdx.x / a.nshots;
  const int x0 = (tile % a.ntx) * TX;
  const int z0 = (tile / a.ntx) * TZ;
  const long long base = (long long)b * a.sstride;
  constexpr int UCH = SROW / 4;
  for (int c = tid; c < (TZ + 2 * HR) * UCH; c += NTHREADS) {
    const int r = c / UCH, cc = c - r * UCH;
    const int z = z0 - HR + r, x = x0 - HX + 4 * cc;
    const int nb = chunk_bytes(z, x, a.nz, a.nx);
    const long long off = (long long)z * a.pitch + x;
    cp_async16(s_u + r * SROW + 4 * cc, nb ? a.u + base + off : a.u, nb);
    cp_async16(s_y + r * SROW + 4 * cc, nb ? a.gy + base + off : a.gy, nb);
    cp_async16(s_k + r * SROW + 4 * cc, nb ? a.k + off : a.k, nb);
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  const int lane = tid & 31, wid = tid >> 5;
  const int xl = 4 * lane;
  const int x = x0 + xl;
  const int sr0 = HR + wid * RPW;
  // centre values of gy before the in-place k*gy
  float4 gyc[RPW];
#pragma unroll
  for (int i = 0; i < RPW; ++i) gyc[i] = lds4(s_y + (sr0 + i) * SROW + HX + xl);
  __syncthreads();
  for (int c = tid; c < (TZ + 2 * HR) * UCH; c += NTHREADS) {
    float4 kk = lds4(s_k + 4 * c);
    const float4 yy = lds4(s_y + 4 * c);
    kk.x *= yy.x; kk.y *= yy.y; kk.z *= yy.z; kk.w *= yy.w;
    sts4(s_y + 4 * c, kk);
  }
  __syncthreads();
  float4 wu[2 * R + 1], wy[2 * R + 1];
#pragma unroll
  for (int j = 0; j < 2 * R; ++j) {
    wu[j] = lds4(s_u + (sr0 - R + j) * SROW + HX + xl);
    wy[j] = lds4(s_y + (sr0 - R + j) * SROW + HX + xl);
  }
#pragma unroll
  for (int i = 0; i < RPW; ++i) {
    const int sr = sr0 + i;
    const int z = z0 + wid * RPW + i;
    wu[2 * R] = lds4(s_u + (sr + R) * SROW + HX + xl);
    wy[2 * R] = lds4(s_y + (sr + R) * SROW + HX + xl);
    const float4 LU = lap4<R>(wu, lds4(s_u + sr * SROW + xl), lds4(s_u + sr * SROW + 2 * HX + xl), a.w);
    const float4 LY = lap4<R>(wy, lds4(s_y + sr * SROW + xl), lds4(s_y + sr * SROW + 2 * HX + xl), a.w);
    if (z < a.nz && x < a.nx) {
      const long long moff = (long long)z * a.pitch + x;
      const long long off = base + moff;
      const float4 vg = *reinterpret_cast<const float4*>(a.g + moff);
      const float4 gy = gyc[i];
      float4 h1 = a.gh1 ? *reinterpret_cast<const float4*>(a.gh1 + off) : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 ou, om;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        set_comp(ou, m, fmaf(comp(vg, m), comp(gy, m), comp(LY, m)) + comp(h1, m));
        set_comp(om, m, (1.f - comp(vg, m)) * comp(gy, m));
        if (x + m < a.nx) {
          const float kk = a.k[moff + m], vv = a.vp[moff + m];
          atomicAdd(a.gvp + moff + m, comp(gy, m) * comp(LU, m) * (2.f * kk / vv));
        }
      }
      *reinterpret_cast<float4*>(a.gu + off) = ou;
      *reinterpret_cast<float4*>(a.gum + off) = om;
    }
#pragma unroll
    for (int j = 0; j < 2 * R; ++j) {
      wu[j] = wu[j + 1];
      wy[j] = wy[j + 1];
    }
  }
}

// ------------------------------------------------------ coefficients ---

__global__ void acoustic_coef_kernel(int nz, int nx, int pitch, const float* __restrict__ vp,
                                     const float* __restrict__ damp, int boundary, float dt, float h,
                                     float* __restrict__ g, float* __restrict__ k) {
  const long long n = (long long)nz * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % pitch);
    if (x >= nx) {
      g[i] = 0.f;
      k[i] = 0.f;
      continue;
    }
    const float q = (boundary == 0 && damp != nullptr) ? damp[i] * dt : 0.f;
    const float v = vp[i];
    const float inv = 1.f / (1.f + q);
    g[i] = 2.f * inv;
    k[i] = (v * v) * (dt * dt) / (h * h) * inv;
  }
}

__global__ void acoustic_grad_reduce_kernel(int nz, int nx, int pitch, int nshots, long long sstride,
                                            const float* __restrict__ grad_shot,
                                            const float* __restrict__ vp, Ring ring,
                                            float* __restrict__ grad_vp) {
  const long long n = (long long)nz * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / pitch), x = (int)(i % pitch);
    float s = 0.f;
    if (x < nx && ring.inside(z, x)) {
      // the adjoint is carried as nu = k * Lambda: dJ/dvp = (2/vp) sum nu L(U)
      for (int b = 0; b < nshots; ++b) s += grad_shot[b * sstride + i];
      if (vp != nullptr) s *= 2.f / vp[i];  // without vp: the sum itself (dJ/dm of Born)
    }
    grad_vp[i] = s;
  }
}

// ------------------------------------------------------------- launch ---

template <int R, int TZ, bool HABC>
static size_t fwd_smem() {
  constexpr int HR = (HABC && R < 2) ? 2 : R;
  return sizeof(float) * ((TZ + 2 * HR) * SROW + TZ * TX) + sizeof(int) * (3 * MAX_TILE_SRC + 1);
}
template <int R, int TZ>
static size_t vjp_smem() {
  return sizeof(float) * (3 * (TZ + 2 * R) * SROW);
}

template <int R, int TZ, bool HABC>
static cudaError_t launch_fwd_t(const AcStepArgs& a, int ntz, cudaStream_t s) {
  const size_t sm = fwd_smem<R, TZ, HABC>();
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(acoustic_fwd_kernel<R, TZ, HABC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long nblk = (long long)a.nshots * a.ntx * ntz;
  acoustic_fwd_kernel<R, TZ, HABC><<<(unsigned)nblk, NTHREADS, sm, s>>>(a);
  return cudaGetLastError();
}

template <int R, int TZ>
static cudaError_t launch_vjp_t(const AcVjpArgs& a, int ntz, cudaStream_t s) {
  const size_t sm = vjp_smem<R, TZ>();
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(acoustic_vjp_kernel<R, TZ>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long nblk = (long long)a.nshots * a.ntx * ntz;
  acoustic_vjp_kernel<R, TZ><<<(unsigned)nblk, NTHREADS, sm, s>>>(a);
  return cudaGetLastError();
}

// Tile height: the tallest tile that still gives >= 2 waves of CTAs.
int pick_tz(int nz, int nx, int nshots, int tz_max) {
  const int ntx = (nx + TX - 1) / TX;
  const long long target = 2LL * 152 * 3;
  for (int tz = tz_max; tz > 8; tz /= 2) {
    const long long n = (long long)nshots * ntx * ((nz + tz - 1) / tz);
    if (n >= target) return tz;
  }
  return 8;
}

template <int TZ, bool HABC>
static cudaError_t fwd_by_r(int R, const AcStepArgs& a, int ntz, cudaStream_t s) {
  switch (R) {
    case 1: return launch_fwd_t<1, TZ, HABC>(a, ntz, s);
    case 2: return launch_fwd_t<2, TZ, HABC>(a, ntz, s);
    case 3: return launch_fwd_t<3, TZ, HABC>(a, ntz, s);
    case 4: return launch_fwd_t<4, TZ, HABC>(a, ntz, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_acoustic_fwd(int R, bool habc, int tz, const AcStepArgs& a, cudaStream_t s) {
  const int ntz = (a.nz + tz - 1) / tz;
  if (habc) {
    if (tz == 32) return fwd_by_r<32, true>(R, a, ntz, s);
    if (tz == 16) return fwd_by_r<16, true>(R, a, ntz, s);
    return fwd_by_r<8, true>(R, a, ntz, s);
  }
  if (tz == 32) return fwd_by_r<32, false>(R, a, ntz, s);
  if (tz == 16) return fwd_by_r<16, false>(R, a, ntz, s);
  return fwd_by_r<8, false>(R, a, ntz, s);
}

cudaError_t launch_acoustic_vjp(int R, const AcVjpArgs& a, cudaStream_t s) {
  constexpr int TZ = 16;
  const int ntz = (a.nz + TZ - 1) / TZ;
  switch (R) {
    case 1: return launch_vjp_t<1, TZ>(a, ntz, s);
    case 2: return launch_vjp_t<2, TZ>(a, ntz, s);
    case 3: return launch_vjp_t<3, TZ>(a, ntz, s);
    case 4: return launch_vjp_t<4, TZ>(a, ntz, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_acoustic_coef(const sgb_grid& gr, const float* vp, const float* damp, int boundary,
                                 float* g, float* k, cudaStream_t s) {
  const long long n = (long long)gr.nz * gr.pitch;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  acoustic_coef_kernel<<<blocks, 256, 0, s>>>(gr.nz, gr.nx, gr.pitch, vp, damp, boundary, gr.dt, gr.h, g, k);
  return cudaGetLastError();
}

cudaError_t launch_acoustic_grad_reduce(const sgb_grid& gr, const float* grad_shot, const float* vp,
                                        const Ring& ring, float* grad_vp, cudaStream_t s) {
  const long long n = (long long)gr.nz * gr.pitch;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  acoustic_grad_reduce_kernel<<<blocks, 256, 0, s>>>(gr.nz, gr.nx, gr.pitch, gr.nshots,
                                                     (long long)gr.nz * gr.pitch, grad_shot, vp, ring, grad_vp);
  return cudaGetLastError();
}

}  // namespace sgb
