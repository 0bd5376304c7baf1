// Fused boundary-saving adjoint step of the acoustic PML equation as a TMA
// tile pipeline (see stream_common.cuh).
//
// The forward step is U_{n+1} = g (U_n - U_{n-1}) + U_{n-1} + k L(U_n) + S w_n
// (acoustic.py:73-86, g = 2/(1+d dt), k = vp^2 dt^2/(h^2 (1+d dt))).  With the
// adjoint Lambda_n = dJ/dU_n, the transposed recursion is
//   Lambda_j = g (L1 - L2) + L2 + L(k L1) + R^T r_{j-1}
// (L1 = Lambda_{j+1}, L2 = Lambda_{j+2}; L is self-adjoint with zero
// padding).  Carrying nu = k Lambda instead gives the forward operator again:
//   nu_j = g (nu1 - nu2) + nu2 + k (L(nu1) + R^T r_{j-1}),
// and dJ/dvp = (2/vp) sum_j nu_j L(U_{j-1}).  One kernel per reverse step:
//   * nu_j from nu_{j+1} (haloed) and nu_{j+2};
//   * the gradient term nu_j L(U_{j-1}) inside the undamped box, added to
//     one gradient plane shared by all shots with 16-byte reduction atomics
//     (the plane stays in L2; per-shot planes cost 8 B of DRAM traffic per
//     shot-point and step);
//   * the reconstruction U_{j-2} = 2 U_{j-1} - (U_j - S w_{j-1}) + k L(U_{j-1})
//     inside the box (g = 2 there), the saved ring around it (each CTA
//     copies a share after its tiles), 0 in the damped band.
#include "stream_common.cuh"

namespace sgb {

// PTM: how the point operands of a tile arrive -- 0: 16-byte global loads
// issued before the stage wait; 1: U_j and nu_{j+2} in the TMA stage (they
// land with the stage, S tiles ahead); 2: also the g and k rows.
template <int R, int TZ, int S, int PTM = 0>
struct BwdTileLayout {
  static constexpr int UW = Row<R>::W;
  static constexpr int UROWS = TZ + 2 * R;
  static constexpr int UF = round32(UROWS * UW);
  static constexpr int PF = TZ * TX;
  static constexpr int PTB = PTM >= 1 ? 2 * PF : 0;  // U_j, nu_{j+2} rows
  static constexpr int CTB = PTM >= 2 ? 2 * PF : 0;  // g, k rows
  static constexpr int STAGE = 2 * UF + PTB + CTB;  // U_{j-1}, nu_{j+1} (haloed), then the point rows
  static constexpr size_t BYTES = (size_t)(S * STAGE + PF) * 4 + S * 8;  // + adjoint-source tile
  static constexpr uint32_t TX_BYTES = (2 * UROWS * UW + PTB + CTB) * 4;
};

template <int R, int TZ, int NWP, int S, int PTM>
__global__ void __launch_bounds__(32 * NWP, TZ / NWP <= 2 ? (PTM >= 2 ? 3 : 4) : 1) acoustic_bwd_tile_kernel(
    const __grid_constant__ CUtensorMap tm_u,     // U_{j-1}   box {W, TZ+2R, 1}
    const __grid_constant__ CUtensorMap tm_n,     // nu_{j+1}  box {W, TZ+2R, 1}
    const __grid_constant__ CUtensorMap tm_up,    // U_j       box {128, TZ, 1} (PTM >= 1)
    const __grid_constant__ CUtensorMap tm_np,    // nu_{j+2}  box {128, TZ, 1} (PTM >= 1)
    const __grid_constant__ CUtensorMap tm_c,     // g, k      box {128, TZ, 2} (PTM == 2)
    const AcBwdStreamArgs a) {
  using Lay = BwdTileLayout<R, TZ, S, PTM>;
  constexpr int RPW = TZ / NWP;
  constexpr int UW = Lay::UW, LO = Row<R>::LO;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* smem = reinterpret_cast<float*>(smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u));
  float* sinj = smem + S * Lay::STAGE;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sinj + Lay::PF);
  __shared__ int s_abort;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int ntiles = a.nshots * a.ntx * a.nzc;
  const int G = gridDim.x;

  auto issue = [&](int t, int stage) {
    const Tile g = tile_geom(t, a.nshots, a.ntx, TZ);
    float* st = smem + stage * Lay::STAGE;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bars[stage], Lay::TX_BYTES);
    tma_load_3d(st, &tm_u, g.x0 - LO, g.z0 - R, g.b, &bars[stage]);
    tma_load_3d(st + Lay::UF, &tm_n, g.x0 - LO, g.z0 - R, g.b, &bars[stage]);
    if constexpr (PTM >= 1) {
      tma_load_3d(st + 2 * Lay::UF, &tm_up, g.x0, g.z0, g.b, &bars[stage]);
      tma_load_3d(st + 2 * Lay::UF + Lay::PF, &tm_np, g.x0, g.z0, g.b, &bars[stage]);
    }
    if constexpr (PTM >= 2) tma_load_3d(st + 2 * Lay::UF + Lay::PTB, &tm_c, g.x0, g.z0, 0, &bars[stage]);
  };
  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
    s_abort = 0;
    for (int s = 0; s < S; ++s)
      if ((int)blockIdx.x + s * G < ntiles) issue(blockIdx.x + s * G, s);
  }
  // the saved ring of U_{j-2}, each CTA a share while its first boxes load:
  // the tiles never write ring cells, and nothing in this launch reads U_{j-2}
  if (a.do_recon && a.ring_in != nullptr)
    ring_copy_share(a.ring, a.nshots, a.pitch, a.sstride, a.uout, const_cast<float*>(a.ring_in), true);
  for (int i = tid; i < Lay::PF / 4; i += 32 * NWP) sts4(sinj + 4 * i, make_float4(0.f, 0.f, 0.f, 0.f));
  __syncthreads();
  int k = 0;
  for (int t = blockIdx.x; t < ntiles; t += G, ++k) {
    const int stage = k % S;
    const Tile g = tile_geom(t, a.nshots, a.ntx, TZ);
    const int x = g.x0 + 4 * lane;
    const bool xin = x < a.nx;
    const int zw = g.z0 + wid * RPW;
    const long long fbase = (long long)g.b * a.sstride;
    // point operands of this warp's rows, issued before the stage wait
    float4 vun[RPW], vn2[RPW], vg[RPW], vk[RPW];
#pragma unroll
    for (int i = 0; i < RPW; ++i) {
      const int z = zw + i;
      vun[i] = vn2[i] = vg[i] = vk[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (xin && z < a.nz) {
        const long long mo = (long long)z * a.pitch + x;
        if constexpr (PTM == 0) {
          vun[i] = ldg4(a.unext + fbase + mo);
          vn2[i] = ldg4(a.n2 + fbase + mo);
        }
        if constexpr (PTM <= 1) {
          vg[i] = ldg4(a.g + mo);
          vk[i] = ldg4(a.k + mo);
        }
      }
    }
    // forward sources of time j-1 in this warp's rows, removed from U_j
    WarpSrc src{0u, -1, 0, 0.f};
    if (a.do_recon && a.src_ptr != nullptr) {
      const int2 zr = __ldg(reinterpret_cast<const int2*>(a.src_zr) + g.b);
      if (zr.x < zw + RPW && zr.y > zw)
        src = warp_sources(lane, g.b, zw, RPW, g.x0, a.src_ptr, a.src_z, a.src_x, a.src_wrow, a.wavelet, a.nt,
                           a.t_src, a.status);
    }
    bool has_rec = false;
    if (a.resid != nullptr) {
      const int2 zr = __ldg(reinterpret_cast<const int2*>(a.rec_zr) + g.b);
      has_rec = zr.x < g.z0 + TZ && zr.y > g.z0;
    }
    // adjoint sources (R^T of the record gather) into the injection tile;
    // every warp zeroes its own rows of it after reading them
    if (has_rec) {
      const int* rp = a.rec_row_ptr + (long long)g.b * a.nz;
      for (int lr = wid; lr < TZ && g.z0 + lr < a.nz; lr += NWP) {
        const int z = g.z0 + lr;
        const int p1 = rp[z + 1];
        for (int q = rp[z] + lane; q < p1; q += 32) {
          const int rx = a.rec_x[q] - g.x0;
          if (rx >= 0 && rx < TX) atomicAdd(sinj + lr * TX + rx, a.resid[(long long)a.rec_col[q] * a.nch]);
        }
      }
      __syncthreads();
    }
    if (!mbar_wait(&bars[stage], (k / S) & 1, a.status)) s_abort = 1;
    const float* st = smem + stage * Lay::STAGE;
    const float* sn = st + Lay::UF;
    const bool cols_all = x >= a.ring.ix0 && x + 3 < a.ring.ix1;
    const bool cols_any = x + 3 >= a.ring.ix0 && x < a.ring.ix1;
    const int lr0 = wid * RPW;
    float4 wu[2 * R + 1], wn[2 * R + 1];
#pragma unroll
    for (int j = 0; j < 2 * R; ++j) {
      wu[j] = lds4(st + (lr0 + j) * UW + LO + 4 * lane);
      wn[j] = lds4(sn + (lr0 + j) * UW + LO + 4 * lane);
    }
    const long long off0 = fbase + (long long)zw * a.pitch + x;
#pragma unroll
    for (int i = 0; i < RPW; ++i) {
      const int lr = lr0 + i;
      const int z = zw + i;
      wu[2 * R] = lds4(st + (lr + 2 * R) * UW + LO + 4 * lane);
      wn[2 * R] = lds4(sn + (lr + 2 * R) * UW + LO + 4 * lane);
      const float4 LU = lap_row<R>(wu, st + (lr + R) * UW, lane, a.w);
      const float4 LN = lap_row<R>(wn, sn + (lr + R) * UW, lane, a.w);
      float4 inj = make_float4(0.f, 0.f, 0.f, 0.f);
      if (has_rec) {
        inj = lds4(sinj + lr * TX + 4 * lane);
        sts4(sinj + lr * TX + 4 * lane, make_float4(0.f, 0.f, 0.f, 0.f));
      }
      const float* sp = st + 2 * Lay::UF + lr * TX + 4 * lane;  // point rows of the stage
      float4 un = PTM >= 1 ? lds4(sp) : vun[i];
      const float4 n2 = PTM >= 1 ? lds4(sp + Lay::PF) : vn2[i];
      const float4 g4 = PTM >= 2 ? lds4(sp + Lay::PTB) : vg[i];
      const float4 k4 = PTM >= 2 ? lds4(sp + Lay::PTB + Lay::PF) : vk[i];
      const float4 n1 = wn[R], u1 = wu[R];
      float4 nj;
      nj.x = fmaf(k4.x, LN.x + inj.x, fmaf(g4.x, n1.x - n2.x, n2.x));
      nj.y = fmaf(k4.y, LN.y + inj.y, fmaf(g4.y, n1.y - n2.y, n2.y));
      nj.z = fmaf(k4.z, LN.z + inj.z, fmaf(g4.z, n1.z - n2.z, n2.z));
      nj.w = fmaf(k4.w, LN.w + inj.w, fmaf(g4.w, n1.w - n2.w, n2.w));
      if (src.mask) apply_sources(src, i, lane, -1.f, un);
      if (z < a.nz && xin) {
        const long long goff = off0 + (long long)i * a.pitch;
        *reinterpret_cast<float4*>(a.lout + goff) = nj;
        const bool zin = z >= a.ring.iz0 && z < a.ring.iz1;
        if (zin && cols_any) {
          float4 gs = make_float4(nj.x * LU.x, nj.y * LU.y, nj.z * LU.z, nj.w * LU.w);
          if (!cols_all) {
#pragma unroll
            for (int m = 0; m < 4; ++m)
              if (x + m < a.ring.ix0 || x + m >= a.ring.ix1) set_comp(gs, m, 0.f);
          }
          red_add4(a.grad_shot + (goff - fbase), gs);
        }
        if (a.do_recon) {
          float4 uo;
          uo.x = fmaf(k4.x, LU.x, fmaf(g4.x, u1.x - un.x, un.x));
          uo.y = fmaf(k4.y, LU.y, fmaf(g4.y, u1.y - un.y, un.y));
          uo.z = fmaf(k4.z, LU.z, fmaf(g4.z, u1.z - un.z, un.z));
          uo.w = fmaf(k4.w, LU.w, fmaf(g4.w, u1.w - un.w, un.w));
          if (zin && cols_all) {
            *reinterpret_cast<float4*>(a.uout + goff) = uo;
          } else {
            // 0 outside the box, ring cells left to the ring scatter below
            const bool zr = z >= a.ring.iz0 - a.ring.rt && z < a.ring.iz1 + a.ring.rb;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
              const int xm = x + m;
              const bool inbox = zin && xm >= a.ring.ix0 && xm < a.ring.ix1;
              const bool ring = !inbox && zr && xm >= a.ring.ix0 - a.ring.rl && xm < a.ring.ix1 + a.ring.rr;
              if (!ring) a.uout[goff + m] = inbox ? comp(uo, m) : 0.f;
            }
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 2 * R; ++j) {
        wu[j] = wu[j + 1];
        wn[j] = wn[j + 1];
      }
    }
    if (__syncthreads_or(s_abort)) break;  // stage free
    if (tid == 0 && t + S * G < ntiles) issue(t + S * G, stage);
  }
  if (s_abort && tid == 0)
    for (int q = k; q < k + S; ++q)
      if ((int)blockIdx.x + q * G < ntiles) mbar_wait(&bars[q % S], (q / S) & 1, nullptr);
}

// ------------------------------------------------------------- launch ---

struct BwdCfg {
  int tz, nwp, s, ptm;
};
static const BwdCfg BWD_TILE_CFGS[] = {{8, 4, 2, 0}, {8, 2, 2, 0}, {16, 4, 2, 0}, {8, 4, 3, 0},
                                       {8, 4, 2, 1}, {8, 4, 2, 2}};

// maps: U_{j-1} and nu_{j+1} stencil boxes, U_j and nu_{j+2} point boxes,
// the coefficient rows (the last three read only by the PTM variants)
template <int R, int TZ, int NWP, int S, int PTM = 0>
static cudaError_t bwd_tile_t(const CUtensorMap* maps, const AcBwdStreamArgs& a, cudaStream_t s) {
  using Lay = BwdTileLayout<R, TZ, S, PTM>;
  const size_t smem = Lay::BYTES + 128;
  auto kern = acoustic_bwd_tile_kernel<R, TZ, NWP, S, PTM>;
  static int blocks = 0;
  if (blocks == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    blocks = resident_blocks(kern, 32 * NWP, smem);
  }
  const int tiles = a.nshots * a.ntx * a.nzc;
  kern<<<(unsigned)(tiles < blocks ? tiles : blocks), 32 * NWP, smem, s>>>(maps[0], maps[1], maps[2], maps[3],
                                                                             maps[4], a);
  return cudaGetLastError();
}

template <int R>
static cudaError_t bwd_tile_r(const CUtensorMap* maps, const AcBwdStreamArgs& a, cudaStream_t s) {
  switch (g_bwd_cfg) {
    case 0: return bwd_tile_t<R, 8, 4, 2>(maps, a, s);
    case 1: return bwd_tile_t<R, 8, 2, 2>(maps, a, s);
    case 2: return bwd_tile_t<R, 16, 4, 2>(maps, a, s);
    case 3: return bwd_tile_t<R, 8, 4, 3>(maps, a, s);
    case 4: return bwd_tile_t<R, 8, 4, 2, 1>(maps, a, s);
    case 5: return bwd_tile_t<R, 8, 4, 2, 2>(maps, a, s);
  }
  return cudaErrorInvalidValue;
}

int bwd_tile_rows() { return BWD_TILE_CFGS[g_bwd_cfg].tz; }

cudaError_t launch_acoustic_bwd_stream(int R, const CUtensorMap* maps, const AcBwdStreamArgs& a,
                                       cudaStream_t s) {
  switch (R) {
    case 1: return bwd_tile_r<1>(maps, a, s);
    case 2: return bwd_tile_r<2>(maps, a, s);
    case 3: return bwd_tile_r<3>(maps, a, s);
    case 4: return bwd_tile_r<4>(maps, a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace sgb
