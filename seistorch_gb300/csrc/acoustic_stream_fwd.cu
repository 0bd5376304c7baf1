// Forward step of the acoustic PML equation as a TMA tile pipeline (see
// stream_common.cuh): u+ = g (u - u-) + u- + k L(u) (acoustic.py:73-86),
// with source injection (source.py:47-57), receiver sampling (probe.py:42-44),
// the illumination sum and the saving of the input's boundary ring fused in.
#include "habc_blend.cuh"
#include "stream_common.cuh"

namespace sgb {

// Strip neighbours of the HABC blend: the current field from the staged
// stencil box where the cell lies in it, else from global memory; the
// previous field from global memory (L2).
struct StageField {
  const float* su;  // staged box: rows [zt, zt + rows), columns [xt, xt + w)
  int zt, xt, rows, w;
  const float* u;
  const float* um;
  long long base;
  int pitch;
  __device__ __forceinline__ float U(int z, int x) const {
    const int r = z - zt, c = x - xt;
    if (r >= 0 && r < rows && c >= 0 && c < w) return su[r * w + c];
    return __ldg(u + base + (long long)z * pitch + x);
  }
  __device__ __forceinline__ float P(int z, int x) const { return __ldg(um + base + (long long)z * pitch + x); }
};

// The one-way blend of four cells of a row that all take the same single
// side (or none, where b = 0): v = one b + (1 - b) y with one = (2 - lam - mu)
// U0 + (lam + 2 mu) U1 - mu U2 + (lam - 1) P0 - lam P1, lam = 2 c dt / h,
// mu = c^2 dt^2 / h^2 (acoustic_habc.py:79-101), in habc_side's order.
__device__ __forceinline__ float4 blend4(const float4& y, const float4& U0, const float4& U1, const float4& U2,
                                         const float4& P0, const float4& P1, const float4& c, const float4& b,
                                         float lamf, float muf) {
  float4 v;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const float cm = comp(c, m), bm = comp(b, m);
    const float lam = cm * lamf;
    const float mu = cm * cm * muf;
    const float t1 = (2.f - lam - mu) * comp(U0, m);
    const float t2 = (lam + 2.f * mu) * comp(U1, m);
    const float t3 = -mu * comp(U2, m);
    const float t4 = (lam - 1.f) * comp(P0, m);
    const float t5 = -lam * comp(P1, m);
    const float uo = t1 + t2 + t3 + t4 + t5;
    set_comp(v, m, uo * bm + (1.f - bm) * comp(y, m));
  }
  return v;
}

// Which single side every cell of the group x..x+3 in row z takes, under the
// mask precedence and corner diagonals of acoustic_habc.py:167-202 (cells of
// no side have b = 0): 0 top, 1 bottom, 2 left, 3 right, or -1 when the
// group holds a corner, a diagonal or cells of two sides.
__device__ __forceinline__ int group_side(int z, int x, int nz, int nx, int hw, bool mult) {
  const int dB = nz - 1 - z;
  if ((z >= hw || mult) && dB >= hw) {      // rows without a top or bottom strip
    if (x + 3 < nx - hw) return 2;
    if (x >= hw) return 3;
    return -1;
  }
  if (!mult && z < hw && dB >= hw) {
    const int xd = nx - hw + z;              // top-right diagonal
    if (x > z && x + 3 < nx - 1 - z && !(xd >= x && xd <= x + 3)) return 0;
    return -1;
  }
  if (dB < hw && z >= hw) {
    const int xd = hw - 1 - dB;              // bottom-left diagonal
    if (x > dB && x + 3 < nx - 1 - dB && !(xd >= x && xd <= x + 3)) return 1;
  }
  return -1;
}

// Cross-stencil x and z parts (1-D second differences, centre -2 sum c) of
// the 4 columns of a lane, as lap_row.
template <int R>
__device__ __forceinline__ void lap_row_xz(const float4 (&win)[2 * R + 1], const float* srow, int lane,
                                           const FdWeights& w, float4& Lx, float4& Lz) {
  const float4 l = lds4(srow + Row<R>::LO - 4 + 4 * lane);
  const float4 r = lds4(srow + Row<R>::LO + 4 + 4 * lane);
  const float4 c = win[R];
  const float a[12] = {l.x, l.y, l.z, l.w, c.x, c.y, c.z, c.w, r.x, r.y, r.z, r.w};
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

// PT: the previous field travels through the TMA stage (prefetched S-1
// tiles ahead) instead of a global load issued before the stage wait.
// SB: shots per tile; one TMA box carries all SB shots (shot is the box's
// third dimension), the coefficient rows and the tile's barrier are shared.
template <int R, int TZ, int S, bool PT, int SB = 1>
struct FwdTileLayout {
  static constexpr int UW = Row<R>::W;
  static constexpr int UROWS = TZ + 2 * R;
  static constexpr int USHOT = UROWS * UW;  // floats of one shot's stencil box
  static constexpr int UF = round32(SB * USHOT);
  static constexpr int PSHOT = TZ * TX;
  static constexpr int STAGE = UF + (PT ? SB * PSHOT : 0);
  static constexpr size_t BYTES = (size_t)S * STAGE * 4 + S * 8;
  static constexpr uint32_t TX_BYTES = (SB * USHOT + (PT ? SB * PSHOT : 0)) * 4;
};

// Tile providers: the single-grid kernel takes its tensor maps and argument
// block as separate parameters (the argument block stays in the constant
// bank); the batch kernel covers every tile of up to MAXG grids (an uneven
// batch: each group has its own shape, shots, buffers and step), tiles
// numbered group after group from tile0[g].
template <int SB>
struct FwdOne {
  const CUtensorMap* tu;
  const CUtensorMap* tum;
  AcStreamArgs a;
  __device__ __forceinline__ int ntiles() const { return (a.nshots + SB - 1) / SB * a.ntx * a.nzc; }
  __device__ __forceinline__ int group(int) const { return 0; }
  __device__ __forceinline__ int first(int) const { return 0; }
  __device__ __forceinline__ const AcStreamArgs& args(int) const { return a; }
  __device__ __forceinline__ const CUtensorMap* map_u(int) const { return tu; }
  __device__ __forceinline__ const CUtensorMap* map_um(int) const { return tum; }
};

template <int MAXG>
struct FwdMany {
  const AcFwdBatch<MAXG>& B;
  __device__ __forceinline__ int ntiles() const { return B.tile0[B.ngroups]; }
  __device__ __forceinline__ int group(int t) const {
    int gi = 0;
    while (gi + 1 < B.ngroups && t >= B.tile0[gi + 1]) ++gi;
    return gi;
  }
  __device__ __forceinline__ int first(int gi) const { return B.tile0[gi]; }
  __device__ __forceinline__ const AcStreamArgs& args(int gi) const { return B.g[gi]; }
  __device__ __forceinline__ const CUtensorMap* map_u(int gi) const { return &B.tm_u[gi]; }
  __device__ __forceinline__ const CUtensorMap* map_um(int gi) const { return &B.tm_um[gi]; }
};

// per group: map_u = U_n [nshots][nz][nx], box {W, TZ+2R, 1};
//            map_um = U_{n-1}, box {128, TZ, 1} (used when PT)
// HB: 0 PML; HABC with 1 the plain update (plus the Born / viscoacoustic
// additive field), 2 VTI (k Lx + kz Lz), 3 variable density (C D(u)) -- one
// instantiation per equation, so each carries only its own branch
// pre(): work of every thread between the first boxes' issue and the first
// stage wait (their load latency covers it)
struct NoPre {
  __device__ __forceinline__ void operator()() const {}
};
template <int R, int TZ, int NWP, int S, bool PT, int SB, class P, int HB = 0, class Pre = NoPre>
__device__ __forceinline__ void fwd_tiles(const P& prov, const Pre& pre = Pre{}) {
  static_assert(SB == 1 || PT, "several shots per tile need the previous field in the stage");
  static_assert(HB == 0 || SB == 1, "the HABC family runs one shot per tile (its rows are read for shot b0)");
  using Lay = FwdTileLayout<R, TZ, S, PT, SB>;
  constexpr int RPW = TZ / NWP;
  constexpr int UW = Lay::UW, LO = Row<R>::LO;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* smem = reinterpret_cast<float*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * Lay::STAGE);
  __shared__ int s_abort;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ntiles = prov.ntiles();
  const int G = gridDim.x;

  auto issue = [&](int t, int stage) {
    const int gi = prov.group(t);
    const AcStreamArgs& a = prov.args(gi);
    const Tile g = tile_geom(t - prov.first(gi), (a.nshots + SB - 1) / SB, a.ntx, TZ);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bars[stage], Lay::TX_BYTES);
    tma_load_3d(smem + stage * Lay::STAGE, prov.map_u(gi), g.x0 - LO, g.z0 - R, g.b * SB, &bars[stage]);
    if (PT)
      tma_load_3d(smem + stage * Lay::STAGE + Lay::UF, prov.map_um(gi), g.x0, g.z0, g.b * SB, &bars[stage]);
  };
  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
    s_abort = 0;
    for (int s = 0; s < S; ++s)
      if ((int)blockIdx.x + s * G < ntiles) issue(blockIdx.x + s * G, s);
  }
  pre();
  __syncthreads();
  int k = 0;
  for (int t = blockIdx.x; t < ntiles; t += G, ++k) {
    const int stage = k % S;
    const int gi = prov.group(t);
    const AcStreamArgs& a = prov.args(gi);
    const Tile g = tile_geom(t - prov.first(gi), (a.nshots + SB - 1) / SB, a.ntx, TZ);
    const int x = g.x0 + 4 * lane;
    const bool xin = x < a.nx;
    const int zw = g.z0 + wid * RPW;  // first row of this warp
    const int b0 = g.b * SB;          // first shot of the tile
    // point operands of this warp's rows, issued before the stage wait (the
    // coefficient rows serve every shot of the tile)
    float4 vm[RPW], vg[RPW], vk[RPW];
    float4 vkz[HB == 2 ? RPW : 1];  // VTI: the kz rows as well
    float4 vrc[HB == 3 ? RPW : 1][5];  // variable density: the C, bx+, bx-, bz+, bz- rows
    // plain HABC equation with an additive field (the Born scattered step,
    // the viscoacoustic term): its rows; else the Born background's m rows
    float4 vbn[HB == 1 ? RPW : 1];
    const float* bnp = nullptr;
    if constexpr (HB == 1) bnp = a.born_in != nullptr ? a.born_in + (long long)b0 * a.sstride : a.born_m;
#pragma unroll
    for (int i = 0; i < RPW; ++i) {
      const int z = zw + i;
      if (xin && z < a.nz) {
        const long long mo = (long long)z * a.pitch + x;
        if (!PT) vm[i] = ldg4(a.um + (long long)b0 * a.sstride + mo);
        vg[i] = ldg4(a.g + mo);
        vk[i] = ldg4(a.k + mo);
        if constexpr (HB == 2) vkz[i] = ldg4(a.kz + mo);
        if constexpr (HB == 1) vbn[i] = (bnp != nullptr && (a.born_in != nullptr || a.born_out != nullptr))
                                            ? ldg4(bnp + mo) : make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (HB == 3) {
#pragma unroll
          for (int q = 0; q < 5; ++q) vrc[i][q] = ldg4(a.rho_c + q * (long long)a.nz * a.pitch + mo);
        }
      } else {
        vm[i] = vg[i] = vk[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (HB == 2) vkz[i] = vm[i];
        if constexpr (HB == 1) vbn[i] = vm[i];
        if constexpr (HB == 3) {
#pragma unroll
          for (int q = 0; q < 5; ++q) vrc[i][q] = vm[i];
        }
      }
    }
    // source rows of the tile's shots, read before the stage wait as well
    int2 szr[SB];
#pragma unroll
    for (int sb = 0; sb < SB; ++sb) {
      szr[sb] = make_int2(0, 0);
      if (a.src_ptr != nullptr && b0 + sb < a.nshots) szr[sb] = __ldg(reinterpret_cast<const int2*>(a.src_zr) + b0 + sb);
    }
    unsigned rec_shots = 0;  // bit sb: shot b0 + sb has receivers in this band
    if (a.records != nullptr) {
#pragma unroll
      for (int sb = 0; sb < SB; ++sb) {
        if (b0 + sb >= a.nshots) break;
        const int2 zr = __ldg(reinterpret_cast<const int2*>(a.rec_zr) + b0 + sb);
        if (zr.x < g.z0 + TZ && zr.y > g.z0) rec_shots |= 1u << sb;
      }
    }
    if (!mbar_wait(&bars[stage], (k / S) & 1, a.status)) s_abort = 1;
    const float* st = smem + stage * Lay::STAGE;
    const int lr0 = wid * RPW;
#pragma unroll
    for (int sb = 0; sb < SB; ++sb) {
      const int b = b0 + sb;
      if (b >= a.nshots) break;
      const long long fbase = (long long)b * a.sstride;
      const float* su = st + sb * Lay::USHOT;
      if (PT) {
#pragma unroll
        for (int i = 0; i < RPW; ++i) vm[i] = lds4(st + Lay::UF + sb * Lay::PSHOT + (lr0 + i) * TX + 4 * lane);
      }
      WarpSrc src{0u, -1, 0, 0.f};
      if (a.src_ptr != nullptr && szr[sb].x < zw + RPW && szr[sb].y > zw)
        src = warp_sources(lane, b, zw, RPW, g.x0, a.src_ptr, a.src_z, a.src_x, a.src_wrow, a.wavelet, a.nt, a.t,
                           a.status);
      float4 win[2 * R + 1];
#pragma unroll
      for (int j = 0; j < 2 * R; ++j) win[j] = lds4(su + (lr0 + j) * UW + LO + 4 * lane);
      float* outp = a.un + fbase + (long long)zw * a.pitch + x;
#pragma unroll
      for (int i = 0; i < RPW; ++i) {
        const int lr = lr0 + i;
        const int z = zw + i;
        win[2 * R] = lds4(su + (lr + 2 * R) * UW + LO + 4 * lane);
        const float* srow = su + (lr + R) * UW;
        const float4 c = win[R];
        float4 y;
        if constexpr (HB == 3 && R == 1) {  // variable density: g (u - u-) + u- + C D(u)
          const int ii = HB == 3 ? i : 0;
          const float4 C4 = vrc[ii][0], bxp = vrc[ii][1], bxn = vrc[ii][2], bzp = vrc[ii][3], bzn = vrc[ii][4];
          const float xs[6] = {srow[LO - 1 + 4 * lane], c.x, c.y, c.z, c.w, srow[LO + 4 + 4 * lane]};
#pragma unroll
          for (int m = 0; m < 4; ++m) {
            const float cc = xs[m + 1];
            const float D = comp(bxp, m) * (xs[m + 2] - cc) - comp(bxn, m) * (cc - xs[m]) +
                            comp(bzp, m) * (comp(win[R + 1], m) - cc) - comp(bzn, m) * (cc - comp(win[R - 1], m));
            set_comp(y, m, fmaf(comp(C4, m), D, fmaf(comp(vg[i], m), cc - comp(vm[i], m), comp(vm[i], m))));
          }
        } else if constexpr (HB == 2) {  // VTI: k Lx + kz Lz
          float4 Lx, Lz;
          lap_row_xz<R>(win, srow, lane, a.w, Lx, Lz);
          const float4 vz = vkz[HB == 2 ? i : 0];
#pragma unroll
          for (int m = 0; m < 4; ++m)
            set_comp(y, m, fmaf(comp(vk[i], m), comp(Lx, m), fmaf(comp(vz, m), comp(Lz, m),
                                                                 fmaf(comp(vg[i], m), comp(c, m) - comp(vm[i], m),
                                                                      comp(vm[i], m)))));
        } else {
          const float4 L = lap_row<R>(win, srow, lane, a.w);
          y.x = fmaf(vk[i].x, L.x, fmaf(vg[i].x, c.x - vm[i].x, vm[i].x));
          y.y = fmaf(vk[i].y, L.y, fmaf(vg[i].y, c.y - vm[i].y, vm[i].y));
          y.z = fmaf(vk[i].z, L.z, fmaf(vg[i].z, c.z - vm[i].z, vm[i].z));
          y.w = fmaf(vk[i].w, L.w, fmaf(vg[i].w, c.w - vm[i].w, vm[i].w));
          if (HB == 1 && (a.born_out != nullptr || a.born_in != nullptr) && xin && z < a.nz) {
            const long long po = (long long)z * a.pitch + x;
            const float4 pre = vbn[HB == 1 ? i : 0];
            if (a.born_out != nullptr) {  // m k L(u): the scattered field's source (Born)
              const float4 mm = a.born_in == nullptr ? pre : ldg4(a.born_m + po);
              *reinterpret_cast<float4*>(a.born_out + fbase + po) =
                  make_float4(mm.x * (vk[i].x * L.x), mm.y * (vk[i].y * L.y), mm.z * (vk[i].z * L.z),
                              mm.w * (vk[i].w * L.w));
            }
            if (a.born_in != nullptr) {
              const float4 sb4 = pre;
              y = make_float4(y.x + sb4.x, y.y + sb4.y, y.z + sb4.z, y.w + sb4.w);
            }
          }
        }
        if (HB != 0 && z < a.nz && xin && (z < a.hw || z >= a.nz - a.hw || x < a.hw || x + 3 >= a.nx - a.hw)) {
          // the one-way blend on strip cells: four cells of one side at once,
          // else cell by cell (corners, diagonals, mixed groups; one copy of
          // its code, not unrolled)
          const int side = (x + 3 < a.nx) ? group_side(z, x, a.nz, a.nx, a.hw, a.multiple != 0) : -1;
          const long long ro = (long long)z * a.pitch + x;
          if (side >= 0) {
            const float4 cv = ldg4(a.vp + ro), bv = ldg4(a.hb + ro);
            float4 U1, U2, P1;
            if (side <= 1) {
              const int dz = side == 0 ? 1 : -1;
              auto urow = [&](int zz) -> float4 {
                const int r = zz - (g.z0 - R);
                return (r >= 0 && r < TZ + 2 * R) ? lds4(su + r * UW + LO + 4 * lane)
                                                  : ldg4(a.u + fbase + (long long)zz * a.pitch + x);
              };
              U1 = urow(z + dz);
              U2 = urow(z + 2 * dz);
              P1 = ldg4(a.um + fbase + ro + dz * (long long)a.pitch);
            } else if (side == 2) {
              const float4 r4 = lds4(srow + LO + 4 + 4 * lane);
              U1 = make_float4(c.y, c.z, c.w, r4.x);
              U2 = make_float4(c.z, c.w, r4.x, r4.y);
              P1 = make_float4(vm[i].y, vm[i].z, vm[i].w, __ldg(a.um + fbase + ro + 4));
            } else {
              const float4 l4 = lds4(srow + LO - 4 + 4 * lane);
              U1 = make_float4(l4.w, c.x, c.y, c.z);
              U2 = make_float4(l4.z, l4.w, c.x, c.y);
              P1 = make_float4(__ldg(a.um + fbase + ro - 1), vm[i].x, vm[i].y, vm[i].z);
            }
            y = blend4(y, c, U1, U2, vm[i], P1, cv, bv, a.lamf, a.muf);
          } else {
            const StageField T{su, g.z0 - R, g.x0 - LO, TZ + 2 * R, UW, a.u, a.um, fbase, a.pitch};
#pragma unroll 1
            for (int m = 0; m < 4; ++m)
              if (x + m < a.nx) set_comp(y, m, habc_point(T, a, z, x + m, comp(y, m)));
          }
        }
        if (src.mask) apply_sources(src, i, lane, 1.f, y);
        if (z < a.nz && xin) {
          *reinterpret_cast<float4*>(outp) = y;
          if (a.illum != nullptr) {
#pragma unroll
            for (int m = 0; m < 4; ++m)
              if (x + m < a.nx) atomicAdd(a.illum + (long long)z * a.pitch + x + m, comp(y, m) * comp(y, m));
          }
        }
        outp += a.pitch;
#pragma unroll
        for (int j = 0; j < 2 * R; ++j) win[j] = win[j + 1];
      }
    }
    // stage free; this tile's outputs visible to the CTA; abort is uniform
    if (__syncthreads_or(s_abort)) break;
    if (tid == 0 && t + S * G < ntiles) issue(t + S * G, stage);
    for (int sb = 0; sb < SB; ++sb) {
      if (!(rec_shots & (1u << sb))) continue;
      const int b = b0 + sb;
      const long long fbase = (long long)b * a.sstride;
      const int* rp = a.rec_row_ptr + (long long)b * a.nz;
      for (int lr = wid; lr < TZ && g.z0 + lr < a.nz; lr += NWP) {
        const int z = g.z0 + lr;
        const int p1 = rp[z + 1];
        for (int q = rp[z] + lane; q < p1; q += 32) {
          const int rx = a.rec_x[q];
          if (rx >= g.x0 && rx < g.x0 + TX)
            a.records[(long long)a.rec_col[q] * a.nch] = a.un[fbase + (long long)z * a.pitch + rx];
        }
      }
    }
  }
  // drain: wait (bounded) for the boxes this CTA issued but did not consume
  if (s_abort && tid == 0)
    for (int q = k; q < k + S; ++q)
      if ((int)blockIdx.x + q * G < ntiles) mbar_wait(&bars[q % S], (q / S) & 1, nullptr);
}

// the second-order HABC instantiations with two rows per warp run 640
// threads per SM (registers held to 102), the others, and the PML ones, 512
// (128 registers)
template <int R, int TZ, int NWP, int S, bool PT, int SB, int HB = 0>
__global__ void __launch_bounds__(32 * NWP, HB != 0 ? ((R == 1 && TZ / NWP <= 2) ? 20 : 16) / NWP : 16 / NWP)
    acoustic_fwd_tile_kernel(const __grid_constant__ CUtensorMap tm_u,
                                                                     const __grid_constant__ CUtensorMap tm_um,
                                                                     const AcStreamArgs a) {
  // the input field's boundary ring for the adjoint, each CTA a share while
  // its first boxes load (the input is read-only in this launch)
  auto ring = [&]() {
    if (a.ring_dst != nullptr)
      ring_copy_share(a.ring, a.nshots, a.pitch, a.sstride, const_cast<float*>(a.ring_src), a.ring_dst, false);
  };
  fwd_tiles<R, TZ, NWP, S, PT, SB, FwdOne<SB>, HB>(FwdOne<SB>{&tm_u, &tm_um, a}, ring);
}

template <int R, int TZ, int NWP, int S, bool PT, int MAXG>
__global__ void __launch_bounds__(32 * NWP) acoustic_fwd_batch_kernel(const __grid_constant__ AcFwdBatch<MAXG> B) {
  fwd_tiles<R, TZ, NWP, S, PT, 1>(FwdMany<MAXG>{B});
}

// ------------------------------------------------------------- launch ---

struct FwdCfg {
  int tz, nwp, s, sb;
};
static const FwdCfg FWD_TILE_CFGS[] = {{16, 4, 3, 1}, {16, 4, 3, 1}, {8, 4, 4, 1},
                                       {32, 8, 2, 1}, {16, 4, 2, 1}, {8, 4, 3, 1}};

// Launches the variant on batch b; with s == nullptr and prepare_only it
// only sets the kernel's shared-memory attribute (done once per variant, and
// before any stream capture).
template <int R, int TZ, int NWP, int S, bool PT, int MAXG, int SB = 1, int HB = 0>
static cudaError_t fwd_tile_t(const AcFwdBatch<MAXG>& b, cudaStream_t s, bool prepare_only) {
  using Lay = FwdTileLayout<R, TZ, S, PT, MAXG == 1 ? SB : 1>;
  const size_t smem = Lay::BYTES + 128;  // + alignment slack
  static int blocks = 0;
  if constexpr (MAXG == 1) {
    auto kern = acoustic_fwd_tile_kernel<R, TZ, NWP, S, PT, SB, HB>;
    if (blocks == 0) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      blocks = resident_blocks(kern, 32 * NWP, smem);
    }
    if (prepare_only) return cudaSuccess;
    const AcStreamArgs& a = b.g[0];
    const int tiles = (a.nshots + SB - 1) / SB * a.ntx * a.nzc;
    if (tiles <= 0) return cudaSuccess;
    kern<<<(unsigned)(tiles < blocks ? tiles : blocks), 32 * NWP, smem, s>>>(b.tm_u[0], b.tm_um[0], b.g[0]);
  } else {
    auto kern = acoustic_fwd_batch_kernel<R, TZ, NWP, S, PT, MAXG>;
    if (blocks == 0) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      blocks = resident_blocks(kern, 32 * NWP, smem);
    }
    if (prepare_only) return cudaSuccess;
    const int tiles = b.tile0[b.ngroups];
    if (tiles <= 0) return cudaSuccess;
    kern<<<(unsigned)(tiles < blocks ? tiles : blocks), 32 * NWP, smem, s>>>(b);
  }
  return cudaGetLastError();
}

template <int R, int MAXG>
static cudaError_t fwd_tile_r(const AcFwdBatch<MAXG>& b, cudaStream_t s, bool prep) {
  switch (g_fwd_cfg) {
    case 0: return fwd_tile_t<R, 16, 4, 3, false>(b, s, prep);
    case 1: return fwd_tile_t<R, 16, 4, 3, true>(b, s, prep);
    case 2: return fwd_tile_t<R, 8, 4, 4, true>(b, s, prep);
    case 3: return fwd_tile_t<R, 32, 8, 2, true>(b, s, prep);
    case 4: return fwd_tile_t<R, 16, 4, 2, true>(b, s, prep);
    case 5: return fwd_tile_t<R, 8, 4, 3, true>(b, s, prep);
  }
  return cudaErrorInvalidValue;
}

template <int MAXG>
static cudaError_t fwd_dispatch(int R, const AcFwdBatch<MAXG>& b, cudaStream_t s, bool prep) {
  switch (R) {
    case 1: return fwd_tile_r<1>(b, s, prep);
    case 2: return fwd_tile_r<2>(b, s, prep);
    case 3: return fwd_tile_r<3>(b, s, prep);
    case 4: return fwd_tile_r<4>(b, s, prep);
  }
  return cudaErrorInvalidValue;
}

int fwd_tile_rows() { return FWD_TILE_CFGS[g_fwd_cfg].tz; }
int fwd_tile_shots() { return FWD_TILE_CFGS[g_fwd_cfg].sb; }
int stencil_box_width(int R) { return (R % 2 == 0) ? TX + 8 : TX + 16; }

// The HABC family's forward: HT-row tiles, 4 warps, HS stages, previous
// field through the TMA stage (the fastest of the variants timed on the
// 64-shot 500 x 1100 second-order grid: 137 us a step against 153-166 us);
// the second-order plain equation (also Born and the viscoacoustic additive
// field) can take any of the HABC_FWD variants (rows per tile, warps,
// stages, previous field via TMA).
constexpr int HT = 8, HS = 3;
struct HabcFwdCfg {
  int tz, nw, s;
  bool pt;
};
constexpr HabcFwdCfg HABC_FWD[6] = {{8, 4, 3, true},   {16, 4, 2, true}, {16, 4, 3, true},
                                    {8, 4, 4, false}, {16, 4, 3, false}, {32, 8, 2, true}};
int habc_tile_rows(int R, int hb) { return (R == 1 && hb == 1) ? HABC_FWD[g_habc_fwd_cfg].tz : HT; }

cudaError_t launch_acoustic_fwd_stream(int R, const CUtensorMap* maps, const AcStreamArgs& a, cudaStream_t s,
                                       bool habc) {
  AcFwdBatch<1> b;
  b.tm_u[0] = maps[0];
  b.tm_um[0] = maps[1];
  b.g[0] = a;
  b.ngroups = 1;
  b.tile0[0] = 0;
  b.tile0[1] = a.nshots * a.ntx * a.nzc;
  if (!habc) return fwd_dispatch<1>(R, b, s, false);
  // variable density and VTI are second order (the reference's kernels)
  if (a.rho_c != nullptr) return R == 1 ? fwd_tile_t<1, HT, 4, HS, true, 1, 1, 3>(b, s, false) : cudaErrorInvalidValue;
  if (a.kz != nullptr) return R == 1 ? fwd_tile_t<1, HT, 4, HS, true, 1, 1, 2>(b, s, false) : cudaErrorInvalidValue;
  switch (R) {
    case 1:
      switch (g_habc_fwd_cfg) {
        case 0: return fwd_tile_t<1, 8, 4, 3, true, 1, 1, 1>(b, s, false);
        case 1: return fwd_tile_t<1, 16, 4, 2, true, 1, 1, 1>(b, s, false);
        case 2: return fwd_tile_t<1, 16, 4, 3, true, 1, 1, 1>(b, s, false);
        case 3: return fwd_tile_t<1, 8, 4, 4, false, 1, 1, 1>(b, s, false);
        case 4: return fwd_tile_t<1, 16, 4, 3, false, 1, 1, 1>(b, s, false);
        case 5: return fwd_tile_t<1, 32, 8, 2, true, 1, 1, 1>(b, s, false);
      }
      return cudaErrorInvalidValue;
    case 2: return fwd_tile_t<2, HT, 4, HS, true, 1, 1, 1>(b, s, false);
    case 3: return fwd_tile_t<3, HT, 4, HS, true, 1, 1, 1>(b, s, false);
    case 4: return fwd_tile_t<4, HT, 4, HS, true, 1, 1, 1>(b, s, false);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_acoustic_fwd_batch(int R, const AcFwdBatch<MAX_BATCH_GROUPS>& b, cudaStream_t s) {
  return fwd_dispatch<MAX_BATCH_GROUPS>(R, b, s, false);
}

cudaError_t prepare_acoustic_fwd_batch(int R) {
  AcFwdBatch<MAX_BATCH_GROUPS> b;
  b.ngroups = 0;
  b.tile0[0] = 0;
  return fwd_dispatch<MAX_BATCH_GROUPS>(R, b, nullptr, true);
}

}  // namespace sgb
