// Isotropic elastic velocity-stress kernels (elastic.py:7-37): the forward
// step with sources / receivers / boundary ring fused in, and the fused
// reverse step (boundary-saving reconstruction + exact discrete adjoint +
// gradient terms), plus the coefficient and chain-rule kernels.
//
// Work decomposition: one warp owns (shot, strip of 120 output columns,
// band of TZ rows) and walks down z keeping the rows it still needs in
// registers, so every field row is read from HBM once per warp.  Lanes hold
// 4 adjacent columns (float4); x neighbours come from the adjacent lane by
// shuffle.  A warp loads 128 columns starting 4 left of its strip, so lanes
// 0 and 31 hold the x halo: the staggered step is two dependent one-cell
// stencils (stresses from velocities, then velocities from the new
// stresses), and the halo lanes make the first stencil's values exact one
// column beyond the strip without any extra code path.  The one-cell
// differences are zero on the first / last row / column (diff_using_roll,
// equations2d/utils.py:3-48); those edges are applied with selects, never by
// multiplying with 0, so whatever sits in the padding columns never leaks in.
#include <cmath>

#include "sgb_common.cuh"
#include "elastic_args.cuh"

namespace sgb {
namespace {

constexpr unsigned FULLM = 0xffffffffu;

__device__ __forceinline__ float4 f4(float a) { return make_float4(a, a, a, a); }
__device__ __forceinline__ float4 operator+(const float4& a, const float4& b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 operator-(const float4& a, const float4& b) {
  return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 operator*(const float4& a, const float4& b) {
  return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w);
}
__device__ __forceinline__ float4 operator*(float s, const float4& b) {
  return make_float4(s * b.x, s * b.y, s * b.z, s * b.w);
}
// a + b * c
__device__ __forceinline__ float4 fma4(const float4& b, const float4& c, const float4& a) {
  return make_float4(fmaf(b.x, c.x, a.x), fmaf(b.y, c.y, a.y), fmaf(b.z, c.z, a.z), fmaf(b.w, c.w, a.w));
}
// components whose bit is set in m, 0 elsewhere
__device__ __forceinline__ float4 sel(unsigned m, const float4& v) {
  return make_float4((m & 1u) ? v.x : 0.f, (m & 2u) ? v.y : 0.f, (m & 4u) ? v.z : 0.f, (m & 8u) ? v.w : 0.f);
}
// per component: bit set -> a, else b
__device__ __forceinline__ float4 pick(unsigned m, const float4& a, const float4& b) {
  return make_float4((m & 1u) ? a.x : b.x, (m & 2u) ? a.y : b.y, (m & 4u) ? a.z : b.z, (m & 8u) ? a.w : b.w);
}
// value at column x - 1 / x + 1 of every component
__device__ __forceinline__ float4 at_left(const float4& v) {
  const float w = __shfl_up_sync(FULLM, v.w, 1);
  return make_float4(w, v.x, v.y, v.z);
}
__device__ __forceinline__ float4 at_right(const float4& v) {
  const float x = __shfl_down_sync(FULLM, v.x, 1);
  return make_float4(v.y, v.z, v.w, x);
}

// Lane geometry of a warp strip.
struct ElLane {
  int lane, x0, xl;   // strip start, first column of this lane
  bool ld;            // columns inside [0, pitch): load
  bool own;           // lanes 1..30 inside [0, nx): write
  unsigned xm;        // bit m: column xl+m >= 1       (x - 1 exists)
  unsigned xp;        // bit m: column xl+m <= nx - 2  (x + 1 exists)
};

__device__ __forceinline__ ElLane make_lane(int x0, int nx, int pitch) {
  ElLane L;
  L.lane = threadIdx.x & 31;
  L.x0 = x0;
  L.xl = x0 - 4 + 4 * L.lane;
  L.ld = L.xl >= 0 && L.xl < pitch;
  L.own = L.lane >= 1 && L.lane <= 30 && L.xl < nx;
  L.xm = 0;
  L.xp = 0;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    if (L.xl + m >= 1) L.xm |= 1u << m;
    if (L.xl + m <= nx - 2) L.xp |= 1u << m;
  }
  return L;
}

// Dx- f = f(x) - f(x-1), Dx+ f = f(x+1) - f(x), zero where the neighbour
// is outside the grid, and their transposes.
__device__ __forceinline__ float4 dxm(const float4& f, const ElLane& L) { return sel(L.xm, f - at_left(f)); }
__device__ __forceinline__ float4 dxp(const float4& f, const ElLane& L) { return sel(L.xp, at_right(f) - f); }
// (Dx-)^T g = [x >= 1] g(x) - [x <= nx-2] g(x+1)
__device__ __forceinline__ float4 dxm_t(const float4& g, const ElLane& L) {
  return sel(L.xm, g) - sel(L.xp, at_right(g));
}
// (Dx+)^T g = [x >= 1] g(x-1) - [x <= nx-2] g(x)
__device__ __forceinline__ float4 dxp_t(const float4& g, const ElLane& L) {
  return sel(L.xm, at_left(g)) - sel(L.xp, g);
}

struct RowIO {
  int nz, pitch;
  __device__ __forceinline__ float4 ld(const float* p, int z, const ElLane& L) const {
    if (L.ld && z >= 0 && z < nz) return __ldg(reinterpret_cast<const float4*>(p + (long long)z * pitch + L.xl));
    return f4(0.f);
  }
  __device__ __forceinline__ void st(float* p, int z, const ElLane& L, const float4& v) const {
    if (L.own) *reinterpret_cast<float4*>(p + (long long)z * pitch + L.xl) = v;
  }
};

// Sources of one shot held one per lane (the first 32 points of the shot):
// row, column and this step's wavelet value; only points whose column lies
// in [lo, hi) are kept.
struct WarpPts {
  int z, x;
  float v;
  unsigned any;
};

__device__ __forceinline__ WarpPts load_sources(const ElPoints& p, int b, int z0, int z1, int lo, int hi,
                                                int* status) {
  WarpPts s{-1, 0, 0.f, 0u};
  if (p.src_ptr != nullptr && p.src_fields != 0) {
    const int2 zr = __ldg(reinterpret_cast<const int2*>(p.src_zr) + b);
    if (zr.x < z1 && zr.y > z0) {
      const int p0 = p.src_ptr[b], p1 = p.src_ptr[b + 1];
      const int q = p0 + (threadIdx.x & 31);
      if (q < p1) {
        const int zs = p.src_z[q], xs = p.src_x[q];
        if (zs >= z0 && zs < z1 && xs >= lo && xs < hi) {
          s.z = zs;
          s.x = xs;
          s.v = p.wavelet[(long long)p.src_wrow[q] * p.nt + p.t];
        }
      }
      if (p1 - p0 > 32 && (threadIdx.x & 31) == 0 && status != nullptr) atomicOr(status, DEV_ERR_CAPACITY);
    }
  }
  s.any = __ballot_sync(FULLM, s.z >= 0);
  return s;
}

// v += sign * (sources of row z); sbuf is this warp's 128-float scratch row.
__device__ __forceinline__ void add_sources(const WarpPts& s, int z, float sign, float4& v, float* sbuf,
                                            const ElLane& L) {
  if (s.any == 0u) return;
  const unsigned m = __ballot_sync(FULLM, s.z == z);
  if (m == 0u) return;
  sts4(sbuf + 4 * L.lane, f4(0.f));
  __syncwarp();
  if (s.z == z) sbuf[s.x - (L.x0 - 4)] = s.v;  // points are unique within a shot
  __syncwarp();
  v = fma4(f4(sign), lds4(sbuf + 4 * L.lane), v);
  __syncwarp();
}

// v += dJ/d(records) of channel `ch` for the receivers of row z whose column
// lies in the warp's 128 loaded columns (duplicates add up); p.rec_row_ptr
// points at this shot's row table.
__device__ __forceinline__ void add_residual(const ElPoints& p, const float* resid, int z, int ch,
                                             float4& v, float* sbuf, const ElLane& L) {
  const int r0 = p.rec_row_ptr[z], r1 = p.rec_row_ptr[z + 1];
  if (r1 <= r0) return;
  sts4(sbuf + 4 * L.lane, f4(0.f));
  __syncwarp();
  for (int q = r0 + L.lane; q < r1; q += 32) {
    const int rx = p.rec_x[q] - (L.x0 - 4);
    if (rx >= 0 && rx < 128) atomicAdd(sbuf + rx, resid[(long long)p.rec_col[q] * p.nch + ch]);
  }
  __syncwarp();
  v = v + lds4(sbuf + 4 * L.lane);
  __syncwarp();
}

// records[col][ch] = v at the receivers of row z inside the strip's 120
// output columns.
__device__ __forceinline__ void sample_row(const ElPoints& p, const int* rp, float* records, int z, int ch,
                                           int nx, const float4& v, float* sbuf, const ElLane& L) {
  const int r0 = rp[z], r1 = rp[z + 1];
  if (r1 <= r0) return;
  sts4(sbuf + 4 * L.lane, v);
  __syncwarp();
  for (int q = r0 + L.lane; q < r1; q += 32) {
    const int rx = p.rec_x[q];
    if (rx >= L.x0 && rx < L.x0 + EL_SW && rx < nx) records[(long long)p.rec_col[q] * p.nch + ch] = sbuf[rx - L.x0 + 4];
  }
  __syncwarp();
}

// Columns of this lane inside [lo, hi) as a 4-bit mask.
__device__ __forceinline__ unsigned col_mask(const ElLane& L, int lo, int hi) {
  unsigned m = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (L.xl + k >= lo && L.xl + k < hi) m |= 1u << k;
  return m;
}

// Does this lane hold ring cells of row z (ring cells are the band around
// the box, see Ring)?
__device__ __forceinline__ bool lane_ring_row(const Ring& R, int z, const ElLane& L) {
  if (R.size == 0 || z < R.iz0 - R.rt || z >= R.iz1 + R.rb) return false;
  const int xa = R.ix0 - R.rl, xb = R.ix1 + R.rr;
  if (L.xl + 3 < xa || L.xl >= xb) return false;
  if (z < R.iz0 || z >= R.iz1) return true;
  return (L.xl < R.ix0) || (L.xl + 3 >= R.ix1);
}

// ------------------------------------------------------------ forward ---

// Rows a forward iteration reads, prefetched one iteration ahead: for step
// row z, vx / vz / txz and the five coefficient rows of z + 1, txx / tzz of z.
constexpr int FWD_PRE_ROWS = 10;

template <int TZ>
__global__ void __launch_bounds__(128) elastic_fwd_kernel(const ElFwdArgs a) {
  __shared__ __align__(16) float sbuf_all[4][128];
  // per warp, two slots of the prefetched rows; each lane copies and reads
  // back only its own 16 bytes, so the slots need no warp synchronisation
  __shared__ __align__(16) float pre_all[4][2][FWD_PRE_ROWS][128];
  float* sbuf = sbuf_all[threadIdx.x >> 5];
  float* pre = &pre_all[threadIdx.x >> 5][0][0][0];
  const int gw = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (gw >= a.nshots * a.nstrip * a.nband) return;  // whole warps; no block barrier below
  const int b = gw % a.nshots;
  const int rest = gw / a.nshots;
  const int x0 = (rest % a.nstrip) * EL_SW;
  const int z0 = (rest / a.nstrip) * TZ;
  const int z1 = min(z0 + TZ, a.nz);
  const int nz = a.nz;
  const ElLane L = make_lane(x0, a.nx, a.pitch);
  const RowIO io{a.nz, a.pitch};
  const long long fb = (long long)b * a.sstride;
  const float* vx = a.in[0] + fb;
  const float* vz = a.in[1] + fb;
  const float* txx = a.in[2] + fb;
  const float* tzz = a.in[3] + fb;
  const float* txz = a.in[4] + fb;
  const WarpPts src = load_sources(a.p, b, z0, z1, x0, x0 + EL_SW, a.status);
  bool has_rec = false;
  const int* rp = nullptr;
  if (a.records != nullptr) {
    const int2 zr = __ldg(reinterpret_cast<const int2*>(a.p.rec_zr) + b);
    has_rec = zr.x < z1 && zr.y > z0;
    rp = a.p.rec_row_ptr + (long long)b * nz;
  }

  // prologue: rows z0 - 1 and z0
  const float4 vx_m = io.ld(vx, z0 - 1, L), vz_m = io.ld(vz, z0 - 1, L);
  float4 vx_c = io.ld(vx, z0, L), vz_c = io.ld(vz, z0, L);
  float4 tzz_p = f4(0.f);  // tzz' of row z - 1 (before sources)
  if (z0 >= 1) {
    const float4 E = dxm(vx_m, L), F = vz_c - vz_m;
    const float4 q = io.ld(a.c.q, z0 - 1, L), pa = io.ld(a.c.pa, z0 - 1, L), la = io.ld(a.c.la, z0 - 1, L);
    tzz_p = fma4(pa, F, fma4(la, E, q * io.ld(tzz, z0 - 1, L)));
  }
  float4 q_c = io.ld(a.c.q, z0, L), pa_c = io.ld(a.c.pa, z0, L), la_c = io.ld(a.c.la, z0, L);
  float4 bv_c = io.ld(a.c.bv, z0, L);
  float4 txz_c;  // txz' of row z (before sources)
  {
    const float4 G = dxp(vz_c, L) + (z0 >= 1 ? vx_c - vx_m : f4(0.f));
    txz_c = fma4(io.ld(a.c.ma, z0, L), G, q_c * io.ld(txz, z0, L));
  }

  auto cp_row = [&](float* dst, const float* src, int zz) {
    const bool ok = L.ld && zz >= 0 && zz < nz;
    cp_async16(dst + 4 * L.lane, ok ? src + (long long)zz * a.pitch + L.xl : src, ok ? 16 : 0);
  };
  auto fetch = [&](int slot, int z) {
    float* d = pre + slot * FWD_PRE_ROWS * 128;
    cp_row(d + 0 * 128, vx, z + 1);
    cp_row(d + 1 * 128, vz, z + 1);
    cp_row(d + 2 * 128, txz, z + 1);
    cp_row(d + 3 * 128, a.c.q, z + 1);
    cp_row(d + 4 * 128, a.c.pa, z + 1);
    cp_row(d + 5 * 128, a.c.la, z + 1);
    cp_row(d + 6 * 128, a.c.ma, z + 1);
    cp_row(d + 7 * 128, a.c.bv, z + 1);
    cp_row(d + 8 * 128, txx, z);
    cp_row(d + 9 * 128, tzz, z);
    cp_async_commit();
  };
  fetch(0, z0);
  for (int z = z0; z < z1; ++z) {
    const int zn = z + 1;
    const int slot = (z - z0) & 1;
    if (zn < z1)
      fetch(slot ^ 1, zn);
    else
      cp_async_commit();  // an empty group keeps the wait count uniform
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    const float* r = pre + slot * FWD_PRE_ROWS * 128 + 4 * L.lane;
    const float4 vx_n = lds4(r + 0 * 128), vz_n = lds4(r + 1 * 128), txz_in = lds4(r + 2 * 128);
    const float4 txx_in = lds4(r + 8 * 128), tzz_in = lds4(r + 9 * 128);
    const float4 q_n = lds4(r + 3 * 128), pa_n = lds4(r + 4 * 128), la_n = lds4(r + 5 * 128);
    const float4 ma_n = lds4(r + 6 * 128), bv_n = lds4(r + 7 * 128);
    // stresses of row z (A-8, A-9) and txz' of row z + 1 (A-10)
    const float4 E = dxm(vx_c, L);
    const float4 F = z < nz - 1 ? vz_n - vz_c : f4(0.f);
    const float4 Txx = fma4(pa_c, E, fma4(la_c, F, q_c * txx_in));
    const float4 Tzz = fma4(pa_c, F, fma4(la_c, E, q_c * tzz_in));
    float4 Txz_n = f4(0.f);
    if (zn < nz) Txz_n = fma4(ma_n, dxp(vz_n, L) + (vx_n - vx_c), q_n * txz_in);
    // velocities of row z from the new stresses
    const float4 dvx = dxp(Txx, L) + (z < nz - 1 ? Txz_n - txz_c : f4(0.f));
    const float4 dvz = dxm(txz_c, L) + (z > 0 ? Tzz - tzz_p : f4(0.f));
    float4 o[5] = {fma4(bv_c, dvx, q_c * vx_c), fma4(bv_c, dvz, q_c * vz_c), Txx, Tzz, txz_c};
    // sources after the step (source.py:47-57)
    if (src.any) {
#pragma unroll
      for (int f = 0; f < 5; ++f)
        if (a.p.src_fields & (1 << f)) add_sources(src, z, 1.f, o[f], sbuf, L);
    }
#pragma unroll
    for (int f = 0; f < 5; ++f) io.st(a.out[f] + fb, z, L, o[f]);
    if (has_rec) {
      for (int ch = 0; ch < a.p.nch; ++ch) {
        const int f = a.p.rec_fields[ch];
        const float4 v = f == 0 ? o[0] : f == 1 ? o[1] : f == 2 ? o[2] : f == 3 ? o[3] : o[4];
        sample_row(a.p, rp, a.records, z, ch, a.nx, v, sbuf, L);
      }
    }
    if (a.illum != nullptr && L.own) {
      const int f = a.illum_field;
      const float4 v = f == 0 ? o[0] : f == 1 ? o[1] : f == 2 ? o[2] : f == 3 ? o[3] : o[4];
      float* ip = a.illum + (long long)z * a.pitch + L.xl;
#pragma unroll
      for (int m = 0; m < 4; ++m)
        if (L.xl + m < a.nx) atomicAdd(ip + m, comp(v, m) * comp(v, m));
    }
    if (a.ring_out != nullptr && L.own && lane_ring_row(a.ring, z, L)) {
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int x = L.xl + m;
        const int ri = x < a.nx ? a.ring.index(z, x) : -1;
        if (ri >= 0) {
#pragma unroll
          for (int f = 0; f < 5; ++f)
            a.ring_out[((long long)f * a.nshots + b) * a.ring.size + ri] = comp(o[f], m);
        }
      }
    }
    vx_c = vx_n;
    vz_c = vz_n;
    tzz_p = Tzz;
    txz_c = Txz_n;
    q_c = q_n;
    pa_c = pa_n;
    la_c = la_n;
    bv_c = bv_n;
  }
}

// ------------------------------------------------------------ reverse ---
//
// Reverse step i.  Notation: s' = s_{i+1} (stresses before this step's
// sources are s'' = s' - sources), a = adjoint of s_{i+1}
// (= a_in + receiver residuals), g = bv a_v.
//   reconstruction (box, q = 1): v_i = v' - bv Dv(s''), T_i = T'' - C D(v_i)
//   adjoint:  aT_m = aT + Dv^T g,  av_m = q av,
//             av_new = av_m + D^T (C aT_m),  aT_new = q aT_m
//   gradient: lambda += (aTxx_m + aTzz_m)(Dx- vx_i + Dz+ vz_i)
//             mu     += 2 aTxx_m Dx- vx_i + 2 aTzz_m Dz+ vz_i + aTxz_m (Dx+ vz_i + Dz- vx_i)
//             buoy   += av . Dv(s'')      (times e, -bv/rho in the chain rule)
// A warp walks rows r = z0-1 .. z1: at row r it completes everything that
// needs rows <= r and finishes row r-1 (the Dz+ vz_i, Dz- hxz terms).

// Rows a reverse iteration r reads, prefetched one iteration ahead (index in
// the slot): s0 s1 (v_in in mode 1) s2 s3 a0 a2 a3 a4 of r; s4 a1 of r + 1;
// in mode 1 the three per-shot gradient rows of r.  The coefficient rows
// (shared by all shots, L2-resident) are read with early __ldg instead.  In
// mode 0 (the reverse loop) every shot adds its gradient terms into plane 0
// of each gradient field with 16-byte reduction atomics: the planes stay in
// L2, and the step moves 80 instead of 104 B per shot-point of DRAM traffic.
template <int MODE>
__host__ __device__ constexpr int bwd_pre_rows() { return MODE == 0 ? 10 : 13; }

template <int TZ, int MODE>
__global__ void __launch_bounds__(128) elastic_bwd_kernel(const ElBwdArgs a) {
  __shared__ __align__(16) float sbuf_all[4][128];
  constexpr int BWD_PRE_ROWS = bwd_pre_rows<MODE>();
  extern __shared__ __align__(16) float bwd_pre[];  // [4 warps][2 slots][BWD_PRE_ROWS][128]
  float* sbuf = sbuf_all[threadIdx.x >> 5];
  float* pre = bwd_pre + (threadIdx.x >> 5) * 2 * BWD_PRE_ROWS * 128;
  const int gw = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (gw >= a.nshots * a.nstrip * a.nband) return;
  const int b = gw % a.nshots;
  const int rest = gw / a.nshots;
  const int x0 = (rest % a.nstrip) * EL_SW;
  const int z0 = (rest / a.nstrip) * TZ;
  const int z1 = min(z0 + TZ, a.nz);
  const int nz = a.nz;
  const ElLane L = make_lane(x0, a.nx, a.pitch);
  const RowIO io{a.nz, a.pitch};
  const long long fb = (long long)b * a.sstride;
  const float* S[5];
  const float* A[5];
#pragma unroll
  for (int f = 0; f < 5; ++f) {
    S[f] = a.s_in[f] + fb;
    A[f] = a.a_in[f] + fb;
  }
  // box columns of this lane (mode 1: every column)
  const unsigned boxc = MODE == 0 ? col_mask(L, a.ring.ix0, a.ring.ix1) : 0xFu;
  const WarpPts src = MODE == 0 ? load_sources(a.p, b, z0 - 1, z1 + 2, x0 - 4, x0 + 124, a.status)
                                : WarpPts{-1, 0, 0.f, 0u};
  bool has_rec = false;
  const int* rp = nullptr;
  if (MODE == 0 && a.resid != nullptr) {
    const int2 zr = __ldg(reinterpret_cast<const int2*>(a.p.rec_zr) + b);
    has_rec = zr.x < z1 + 2 && zr.y > z0 - 1;
    rp = a.p.rec_row_ptr + (long long)b * nz;
  }
  ElPoints pr = a.p;
  pr.rec_row_ptr = rp;

  // corrections on loading: this step's sources leave the state (s''), the
  // receiver residuals of the channels on field f enter the adjoint
  auto fix_s = [&](float4 v, int f, int z) {
    if (MODE == 0 && (a.p.src_fields & (1 << f)) && z >= 0 && z < nz) add_sources(src, z, -1.f, v, sbuf, L);
    return v;
  };
  auto fix_a = [&](float4 v, int f, int z) {
    if (MODE == 0 && has_rec && z >= 0 && z < nz) {
      for (int ch = 0; ch < a.p.nch; ++ch)
        if (a.p.rec_fields[ch] == f) add_residual(pr, a.resid, z, ch, v, sbuf, L);
    }
    return v;
  };
  auto lds = [&](int f, int z) { return fix_s(io.ld(S[f], z, L), f, z); };
  auto lda = [&](int f, int z) { return fix_a(io.ld(A[f], z, L), f, z); };
  auto cp_row = [&](float* dst, const float* src, int zz) {
    const bool ok = L.ld && zz >= 0 && zz < nz;
    cp_async16(dst + 4 * L.lane, ok ? src + (long long)zz * a.pitch + L.xl : src, ok ? 16 : 0);
  };
  // v into row z of plane 0 of a gradient field (this lane's four columns)
  auto gred = [&](float* plane, int z, const float4& v) {
    if (L.own) red_add4(plane + (long long)z * a.pitch + L.xl, v);
  };
  auto fetch = [&](int slot, int r) {
    float* d = pre + slot * BWD_PRE_ROWS * 128;
    cp_row(d + 0 * 128, MODE == 0 ? S[0] : a.v_in[0] + fb, r);
    cp_row(d + 1 * 128, MODE == 0 ? S[1] : a.v_in[1] + fb, r);
    cp_row(d + 2 * 128, S[2], r);
    cp_row(d + 3 * 128, S[3], r);
    cp_row(d + 4 * 128, A[0], r);
    cp_row(d + 5 * 128, A[2], r);
    cp_row(d + 6 * 128, A[3], r);
    cp_row(d + 7 * 128, A[4], r);
    cp_row(d + 8 * 128, S[4], r + 1);
    cp_row(d + 9 * 128, A[1], r + 1);
    if (MODE == 1) {
      const bool wrr = r >= z0 && r < z1;  // gradient rows are only read where this warp writes them
      cp_row(d + 10 * 128, a.grad[0] + fb, wrr ? r : -1);
      cp_row(d + 11 * 128, a.grad[1] + fb, wrr ? r : -1);
      cp_row(d + 12 * 128, a.grad[2] + fb, wrr ? r : -1);
    }
    cp_async_commit();
  };
  auto ringv = [&](int f, int z, unsigned m) {  // ring values of s_i for the components in m
    float4 v = f4(0.f);
    if (a.ring_in != nullptr && m != 0u) {
      const float* rb = a.ring_in + ((long long)f * a.nshots + b) * a.ring.size;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (m & (1u << k)) set_comp(v, k, rb[a.ring.index(z, L.xl + k)]);
    }
    return v;
  };
  auto ring_mask = [&](int z) -> unsigned {
    if (MODE != 0 || !lane_ring_row(a.ring, z, L)) return 0u;
    unsigned m = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int x = L.xl + k;
      if (x >= 0 && x < a.nx && a.ring.index(z, x) >= 0) m |= 1u << k;
    }
    return m;
  };

  // carries from row r - 1
  float4 vxi_p = f4(0.f), vzi_p = f4(0.f), hzz_p = f4(0.f), tzz_p = f4(0.f), gx_p = f4(0.f);
  float4 avxpart_p = f4(0.f), txxpart_p = f4(0.f), tzzpart_p = f4(0.f), pa_p = f4(0.f), la_p = f4(0.f);
  float4 S_p = f4(0.f), atzz_p = f4(0.f), glam_p = f4(0.f), gmu_p = f4(0.f);
  // row r parts fetched one row ahead: txz'' (r), av_z (r), g_z (r)
  float4 txz_r = lds(4, z0 - 1);
  float4 avz_r = lda(1, z0 - 1);
  float4 gz_r = io.ld(a.c.bv, z0 - 1, L) * avz_r;

  fetch(0, z0 - 1);
  for (int r = z0 - 1; r <= z1; ++r) {
    const bool inrow = r >= 0 && r < nz;
    const bool wr = r >= z0 && r < z1;
    const bool fin = r - 1 >= z0 && r - 1 < z1;
    const unsigned box = (MODE == 1 || (r >= a.ring.iz0 && r < a.ring.iz1)) ? boxc : 0u;
    const int slot = (r - (z0 - 1)) & 1;
    if (r + 1 <= z1)
      fetch(slot ^ 1, r + 1);
    else
      cp_async_commit();  // an empty group keeps the wait count uniform
    const float4 q = io.ld(a.c.q, r, L), pa = io.ld(a.c.pa, r, L), la = io.ld(a.c.la, r, L);
    const float4 ma = io.ld(a.c.ma, r, L), bv = io.ld(a.c.bv, r, L), bv_n = io.ld(a.c.bv, r + 1, L);
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    const float* pr_ = pre + slot * BWD_PRE_ROWS * 128 + 4 * L.lane;
    // row r
    const float4 txx = fix_s(lds4(pr_ + 2 * 128), 2, r), tzz = fix_s(lds4(pr_ + 3 * 128), 3, r);
    const float4 avx = fix_a(lds4(pr_ + 4 * 128), 0, r);
    const float4 atxx = fix_a(lds4(pr_ + 5 * 128), 2, r), atzz = fix_a(lds4(pr_ + 6 * 128), 3, r);
    const float4 atxz = fix_a(lds4(pr_ + 7 * 128), 4, r);
    // row r + 1 parts
    const float4 txz_n = fix_s(lds4(pr_ + 8 * 128), 4, r + 1);
    const float4 avz_n = fix_a(lds4(pr_ + 9 * 128), 1, r + 1);
    const float4 gz_n = bv_n * avz_n;
    const float4 gx = bv * avx;
    // velocity part: Dv(s'') and v_i
    const float4 dvx = dxp(txx, L) + (r <= nz - 2 ? txz_n - txz_r : f4(0.f));
    const float4 dvz = dxm(txz_r, L) + (r >= 1 ? tzz - tzz_p : f4(0.f));
    float4 vxi, vzi;
    unsigned rmask = 0u;
    if (MODE == 0) {
      rmask = inrow ? ring_mask(r) : 0u;
      const float4 vxs = fix_s(lds4(pr_ + 0 * 128), 0, r), vzs = fix_s(lds4(pr_ + 1 * 128), 1, r);
      vxi = pick(box, vxs - bv * dvx, ringv(0, r, rmask));
      vzi = pick(box, vzs - bv * dvz, ringv(1, r, rmask));
    } else {
      vxi = lds4(pr_ + 0 * 128);
      vzi = lds4(pr_ + 1 * 128);
    }
    const float4 gb_inc = sel(box, fma4(avx, dvx, avz_r * dvz));
    // stress adjoint after the velocity transpose
    const float4 atxx_m = atxx + dxp_t(gx, L);
    const float4 atxz_m = atxz + (r >= 1 ? gx_p : f4(0.f)) - (r <= nz - 2 ? gx : f4(0.f)) + dxm_t(gz_r, L);
    const float4 atzz_m = atzz + (r >= 1 ? gz_r : f4(0.f)) - (r <= nz - 2 ? gz_n : f4(0.f));
    const float4 hxx = fma4(pa, atxx_m, la * atzz_m);
    const float4 hzz = fma4(la, atxx_m, pa * atzz_m);
    const float4 hxz = inrow ? ma * atxz_m : f4(0.f);
    // finish row r - 1
    if (fin) {
      const int zp = r - 1;
      const float4 avx_new = avxpart_p - (inrow ? hxz : f4(0.f));
      const float4 F = zp <= nz - 2 ? vzi - vzi_p : f4(0.f);
      io.st(a.a_out[0] + fb, zp, L, avx_new);
      if (MODE == 0) {
        io.st(a.s_out[2] + fb, zp, L, txxpart_p - la_p * F);
        io.st(a.s_out[3] + fb, zp, L, tzzpart_p - pa_p * F);
      }
      if (MODE == 0) {
        gred(a.grad[0], zp, fma4(S_p, F, glam_p));
        gred(a.grad[1], zp, fma4(2.f * atzz_p, F, gmu_p));
      } else {
        io.st(a.grad[0] + fb, zp, L, fma4(S_p, F, glam_p));
        io.st(a.grad[1] + fb, zp, L, fma4(2.f * atzz_p, F, gmu_p));
      }
    }
    // row r parts that need rows <= r only
    const float4 E = dxm(vxi, L);
    const float4 G = dxp(vzi, L) + (r >= 1 ? vxi - vxi_p : f4(0.f));
    if (wr) {
      const float4 Sx = sel(box, atxx_m + atzz_m);
      // mode 0: the increments only (added to the shared planes); mode 1:
      // the per-shot accumulators
      float4 glam = MODE == 0 ? f4(0.f) : lds4(pr_ + 10 * 128);
      float4 gmu = MODE == 0 ? f4(0.f) : lds4(pr_ + 11 * 128);
      const float4 gbv = MODE == 0 ? gb_inc : lds4(pr_ + 12 * 128) + gb_inc;
      glam = fma4(Sx, E, glam);
      gmu = gmu + sel(box, fma4(2.f * atxx_m, E, atxz_m * G));
      if (MODE == 0) {
        const float4 txz_i = pick(box, txz_r - ma * G, ringv(4, r, rmask));
        txxpart_p = pick(box, txx - pa * E, ringv(2, r, rmask));
        tzzpart_p = pick(box, tzz - la * E, ringv(3, r, rmask));
        io.st(a.s_out[0] + fb, r, L, vxi);
        io.st(a.s_out[1] + fb, r, L, vzi);
        io.st(a.s_out[4] + fb, r, L, txz_i);
      }
      pa_p = sel(box, pa);
      la_p = sel(box, la);
      S_p = Sx;
      atzz_p = sel(box, atzz_m);
      glam_p = glam;
      gmu_p = gmu;
      if (MODE == 0)
        gred(a.grad[2], r, gbv);
      else
        io.st(a.grad[2] + fb, r, L, gbv);
    }
    // adjoint velocities: avz complete, avx waits for hxz(r + 1)
    const float4 avxpart = fma4(q, avx, dxm_t(hxx, L) + (r >= 1 ? hxz : f4(0.f)));
    const float4 avz_new = fma4(q, avz_r, dxp_t(hxz, L) + (r >= 1 ? hzz_p : f4(0.f)) - (r <= nz - 2 ? hzz : f4(0.f)));
    if (wr) {
      io.st(a.a_out[1] + fb, r, L, avz_new);
      io.st(a.a_out[2] + fb, r, L, q * atxx_m);
      io.st(a.a_out[3] + fb, r, L, q * atzz_m);
      io.st(a.a_out[4] + fb, r, L, q * atxz_m);
    }
    avxpart_p = avxpart;
    vxi_p = vxi;
    vzi_p = vzi;
    hzz_p = hzz;
    tzz_p = tzz;
    gx_p = gx;
    txz_r = txz_n;
    avz_r = avz_n;
    gz_r = gz_n;
  }
}

// ------------------------------------------------- setup / reductions ---

__global__ void elastic_coef_kernel(int nz, int nx, int pitch, const float* vp, const float* vs, const float* rho,
                                    const float* d, double dt, double h, float* q, float* e, float* pa, float* la,
                                    float* ma, float* bv) {
  const long long n = (long long)nz * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % pitch);
    if (x >= nx) {
      q[i] = e[i] = pa[i] = la[i] = ma[i] = bv[i] = 0.f;
      continue;
    }
    const double c = 0.5 * dt * (double)d[i];
    const double r = (double)rho[i], p = (double)vp[i], s = (double)vs[i];
    const double lam = r * (p * p - 2.0 * s * s), mu = r * s * s;
    const double ee = dt / (h * (1.0 + c));
    q[i] = (float)((1.0 - c) / (1.0 + c));
    e[i] = (float)ee;
    pa[i] = (float)(ee * (lam + 2.0 * mu));
    la[i] = (float)(ee * lam);
    ma[i] = (float)(ee * mu);
    bv[i] = (float)(ee / r);
  }
}

// grad_out = chain rule of the per-shot lambda / mu / buoyancy terms:
//   dJ/dlambda = e sum_b gl, dJ/dmu = e sum_b gm, dJ/dbv = sum_b gb
//   vp: 2 rho vp dJ/dlambda; vs: -4 rho vs dJ/dlambda + 2 rho vs dJ/dmu;
//   rho: (vp^2 - 2 vs^2) dJ/dlambda + vs^2 dJ/dmu - bv / rho dJ/dbv.
__global__ void elastic_grad_kernel(int nz, int nx, int pitch, int nshots, long long sstride, const float* gl,
                                    const float* gm, const float* gb, const float* e, const float* bv,
                                    const float* vp, const float* vs, const float* rho, int boxed, int iz0, int iz1,
                                    int ix0, int ix1, float* gvp, float* gvs, float* grho) {
  const long long n = (long long)nz * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / pitch), x = (int)(i % pitch);
    float ovp = 0.f, ovs = 0.f, orho = 0.f;
    if (x < nx && (!boxed || (z >= iz0 && z < iz1 && x >= ix0 && x < ix1))) {
      double sl = 0, sm = 0, sb = 0;
      for (int s = 0; s < nshots; ++s) {
        sl += gl[s * sstride + i];
        sm += gm[s * sstride + i];
        sb += gb[s * sstride + i];
      }
      const double dl = (double)e[i] * sl, dm = (double)e[i] * sm;
      const double r = rho[i], p = vp[i], v = vs[i];
      ovp = (float)(2.0 * r * p * dl);
      ovs = (float)(-4.0 * r * v * dl + 2.0 * r * v * dm);
      orho = (float)((p * p - 2.0 * v * v) * dl + v * v * dm - (double)bv[i] / r * sb);
    }
    if (gvp) gvp[i] = ovp;
    if (gvs) gvs[i] = ovs;
    if (grho) grho[i] = orho;
  }
}

// Rows per band: each warp walks one (shot, 120-column strip, band).  Short
// bands (many warps in flight) won on the 400 x 900, 32-shot grid: forward
// 0.62 / 0.71 / 0.74 and reverse 0.57 / 0.62 / 0.60 of measured HBM at
// 32 / 16 / 8 rows (longer bands that fill whole waves lost further).
constexpr int EL_TZ = 16, EL_TZ_FWD = 8, EL_TZ_REV = 16;

template <class K>
void grid_for(K, long long n, int* blocks) {
  long long b = (n + 255) / 256;
  *blocks = (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

}  // namespace

void elastic_strip_geometry(int nz, int nx, int* nstrip, int* nband) {
  *nstrip = (nx + EL_SW - 1) / EL_SW;
  *nband = (nz + EL_TZ - 1) / EL_TZ;
}

cudaError_t launch_elastic_fwd(const ElFwdArgs& a0, cudaStream_t s) {
  ElFwdArgs a = a0;
  a.nband = (a.nz + EL_TZ_FWD - 1) / EL_TZ_FWD;
  const long long warps = (long long)a.nshots * a.nstrip * a.nband;
  elastic_fwd_kernel<EL_TZ_FWD><<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_elastic_bwd(const ElBwdArgs& a0, int mode, cudaStream_t s) {
  ElBwdArgs a = a0;
  a.nband = (a.nz + EL_TZ_REV - 1) / EL_TZ_REV;
  const long long warps = (long long)a.nshots * a.nstrip * a.nband;
  constexpr size_t smem0 = 4 * 2 * bwd_pre_rows<0>() * 128 * sizeof(float);
  constexpr size_t smem1 = 4 * 2 * bwd_pre_rows<1>() * 128 * sizeof(float);
  static bool set = false;
  if (!set) {
    cudaError_t e = cudaFuncSetAttribute(elastic_bwd_kernel<EL_TZ_REV, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem0);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(elastic_bwd_kernel<EL_TZ_REV, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
    if (e != cudaSuccess) return e;
    set = true;
  }
  if (mode == 0)
    elastic_bwd_kernel<EL_TZ_REV, 0><<<(unsigned)((warps + 3) / 4), 128, smem0, s>>>(a);
  else
    elastic_bwd_kernel<EL_TZ_REV, 1><<<(unsigned)((warps + 3) / 4), 128, smem1, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_elastic_coef(const sgb_grid& g, const float* vp, const float* vs, const float* rho,
                                const float* d, float* coef, cudaStream_t s) {
  const long long n = (long long)g.nz * g.pitch;
  int blocks = 0;
  grid_for(0, n, &blocks);
  elastic_coef_kernel<<<blocks, 256, 0, s>>>(g.nz, g.nx, g.pitch, vp, vs, rho, d, (double)g.dt, (double)g.h, coef,
                                             coef + n, coef + 2 * n, coef + 3 * n, coef + 4 * n, coef + 5 * n);
  return cudaGetLastError();
}

cudaError_t launch_elastic_grad(const sgb_grid& g, const float* coef, const float* const gs[3], const float* vp,
                                const float* vs, const float* rho, int boxed, int iz0, int iz1, int ix0, int ix1,
                                float* const out[3], cudaStream_t s) {
  const long long n = (long long)g.nz * g.pitch;
  int blocks = 0;
  grid_for(0, n, &blocks);
  elastic_grad_kernel<<<blocks, 256, 0, s>>>(g.nz, g.nx, g.pitch, g.nshots, n, gs[0], gs[1], gs[2], coef + n,
                                             coef + 5 * n, vp, vs, rho, boxed, iz0, iz1, ix0, ix1, out[0], out[1],
                                             out[2]);
  return cudaGetLastError();
}

}  // namespace sgb
