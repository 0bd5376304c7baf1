// BF16 x BF16 -> FP32 GEMM on the 5th-generation tensor cores (tcgen05) for
// the learned gradient preconditioner's 3x3 convolutions.
//
// One CTA computes a 128 x BN tile of D = sum_k A[m, k] B[n, k] (both
// operands K-major) with the accumulator in tensor memory:
//   warp 0 lane 0  -- TMA producer: per K step one A box (128 rows x RB
//                     bytes) and one B box (BN rows x RB bytes) into a stage
//                     of an S-deep ring, 128/64-byte swizzled;
//   warp 1 lane 0  -- MMA issuer: RB/32 tcgen05.mma (K = 16) per stage, then
//                     tcgen05.commit to the stage's "empty" mbarrier;
//   all 4 warps    -- epilogue: tcgen05.ld of their 32 TMEM lanes (= rows).
// Warp 0 allocates and frees the TMEM columns.  Every wait is bounded; on a
// timeout the CTA records DEV_ERR_TIMEOUT, waits (bounded) for what it
// issued and frees its TMEM before returning.
//
// Two operand modes:
//   CONV  : implicit GEMM of a 3x3 convolution (zero padding 1).  A = input
//           activation NHWC, rows = 128 output pixels (TH rows x TW columns
//           of one image), K step = (tap, 32/64-channel chunk) read at the
//           tap's shifted (x, y) -- shifts are on the W and H dimensions of
//           the tensor map, never on the innermost one; B = weights
//           [Cout][9][Cin].  Used for the forward pass and, with flipped
//           transposed weights, for the data gradient.
//   WGRAD : weight gradient of one tap (blockIdx.z % 9) and 128 output
//           channels (blockIdx.z / 9): A = dY in CHW (rows = output channels), B = the input in CHW shifted by the tap's x
//           offset (one of three pre-shifted copies) and read at the tap's y
//           offset; K = pixels, split over blockIdx.x; FP32 atomics into
//           dW[cout][cin][3][3].
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "sgb_common.cuh"
#include "tma.cuh"
#include "nn_args.cuh"

namespace sgb {
namespace nn {
namespace {

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of a K-major, swizzled operand tile whose
// rows are RB bytes (RB = 128: 128-byte swizzle, RB = 64: 64-byte swizzle);
// 8-row groups are 8 * RB bytes apart.
template <int RB>
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  constexpr uint64_t layout = RB == 128 ? 2ull : 4ull;  // SWIZZLE_128B : SWIZZLE_64B
  constexpr uint64_t sbo = (8ull * RB) >> 4;
  return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | (sbo << 32) | (1ull << 46) | (layout << 61);
}

// Instruction descriptor: D fp32, A and B bf16, both K-major, M = 128, N = BN.
template <int BN>
__device__ __forceinline__ uint32_t instr_desc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int BN, int RB, int S>
struct GemmLayout {
  static constexpr int A_BYTES = 128 * RB;
  static constexpr int B_BYTES = BN * RB;
  static constexpr int STAGE = A_BYTES + B_BYTES;  // multiple of 1024 for every (BN, RB) used
  static constexpr int BYTES = S * STAGE + 1024 /*align*/ + 256 /*barriers + tmem slot*/;
  // two accumulator buffers of at least 32 columns
  static constexpr int ACC_COLS = BN < 32 ? 32 : BN;
  static constexpr int TMEM_COLS = 2 * ACC_COLS;
};

// Tile t of the logical grid and its K range.
struct GemmTile {
  int n_img, y0, x0, m0, tap, n0, kbeg, kend;
};

template <int BN>
__device__ __forceinline__ GemmTile decode_tile(const GemmArgs& g, int t) {
  GemmTile q;
  const int bx = t % g.gx, rest = t / g.gx;
  const int by = rest % g.gy, bz = rest / g.gy;
  q.n0 = by * BN;
  q.kbeg = 0;
  q.kend = g.kiters;
  q.n_img = q.y0 = q.x0 = q.m0 = q.tap = 0;
  if (g.mode == MODE_CONV) {
    const int per_img = g.tiles_x * g.tiles_y;
    q.n_img = bx / per_img;
    const int r = bx % per_img;
    q.y0 = (r / g.tiles_x) * g.TH;
    q.x0 = (r % g.tiles_x) * g.TW;
  } else {
    q.tap = bz % 9;
    q.m0 = (bz / 9) * 128;
    q.kbeg = bx * g.k_per_split;
    q.kend = min(q.kbeg + g.k_per_split, g.kiters);
  }
  return q;
}

// 16-byte store of eight bf16 / four fp32 values
__device__ __forceinline__ void st_bf16x8(__nv_bfloat16* p, const float* v) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    w[i] = *reinterpret_cast<const uint32_t*>(&h);
  }
  *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
}

// Persistent CTA of 192 threads walking the tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ...:
//   warp 0 lane 0  -- TMA producer: per K step one A box (128 rows x RB
//                     bytes) and one B box (BN rows x RB bytes) into the next
//                     stage of an S-deep ring that runs on across tiles;
//   warp 1 lane 0  -- MMA issuer: RB/32 tcgen05.mma (K = 16) per stage into
//                     accumulator buffer (tile & 1), tcgen05.commit to the
//                     stage's "empty" barrier and, after a tile's last stage,
//                     to the buffer's "full" barrier;
//   warps 2..5     -- epilogue: tcgen05.ld of TMEM lanes 32 (warp % 4) ..
//                     +31 (= tile rows) of the finished buffer, then arrive
//                     on its "empty" barrier, so that the MMAs of the next
//                     tile overlap this tile's epilogue.
// Warp 0 allocates and frees the TMEM columns.  Every wait is bounded; on a
// timeout the CTA records DEV_ERR_TIMEOUT, stops, waits (bounded) for the
// copies and MMAs it issued and frees its TMEM before returning.
template <int BN, int RB, int S>
__global__ void __launch_bounds__(192, 1) nn_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB0,
                                                         const __grid_constant__ CUtensorMap tmB1,
                                                         const __grid_constant__ CUtensorMap tmB2,
                                                         const GemmArgs g) {
  using Lay = GemmLayout<BN, RB, S>;
  constexpr int KSTEPS = RB / 32;  // tcgen05.mma K = 16 bf16 = 32 bytes
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + S * Lay::STAGE);
  uint64_t* empty = full + S;
  uint64_t* acc_full = empty + S;  // [2]
  uint64_t* acc_empty = acc_full + 2;  // [2]
  uint64_t* done = acc_empty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  __shared__ int s_fail, s_issued, s_consumed;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = g.gx * g.gy * g.gz;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                 "r"(Lay::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);  // one arrival per epilogue warp
    }
    mbar_init(done, 1);
    fence_mbar_init();
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  volatile int* fail = &s_fail;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer
    int it = 0;  // K steps issued, over all tiles of this CTA
    for (int t = blockIdx.x; t < ntiles && !*fail; t += gridDim.x) {
      const GemmTile q = decode_tile<BN>(g, t);
      const CUtensorMap* tmB = &tmB0;
      if (g.mode == MODE_WGRAD) {
        const int kx = q.tap % 3;
        tmB = kx == 0 ? &tmB0 : (kx == 1 ? &tmB1 : &tmB2);
      }
      for (int k = q.kbeg; k < q.kend; ++k) {
        const int s = it % S;
        if (it >= S && !mbar_wait(&empty[s], ((it / S) - 1) & 1, g.status)) {
          *fail = 1;
          break;
        }
        if (*fail) break;
        unsigned char* sa = base + s * Lay::STAGE;
        unsigned char* sb = sa + Lay::A_BYTES;
        mbar_arrive_expect_tx(&full[s], Lay::STAGE);
        if (g.mode == MODE_CONV) {
          const int tp = k / g.nchunk, c0 = (k % g.nchunk) * (RB / 2);
          const int ky = tp / 3, kx = tp % 3;
          tma_load_4d(sa, &tmA, c0, q.x0 - 1 + kx, q.y0 - 1 + ky, q.n_img, &full[s]);
          tma_load_3d(sb, tmB, c0, tp, q.n0, &full[s]);
        } else {
          const int xc = k % g.wchunks, rest = k / g.wchunks;
          const int y = rest % g.H, n = rest / g.H;
          const int ky = q.tap / 3;
          tma_load_4d(sa, &tmA, xc * 64, y, q.m0, n, &full[s]);
          tma_load_4d(sb, tmB, xc * 64, y - 1 + ky, q.n0, n, &full[s]);
        }
        ++it;
      }
    }
    s_issued = it;
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    const uint32_t idesc = instr_desc<BN>();
    int it = 0, lt = 0;  // K steps consumed, tiles of this CTA
    for (int t = blockIdx.x; t < ntiles && !*fail; t += gridDim.x, ++lt) {
      const GemmTile q = decode_tile<BN>(g, t);
      if (q.kend <= q.kbeg) continue;  // (no such tile: every split has a step)
      const int buf = lt & 1;
      if (lt >= 2 && !mbar_wait(&acc_empty[buf], ((lt >> 1) - 1) & 1, g.status)) {
        *fail = 1;
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(buf * Lay::ACC_COLS);
      for (int k = q.kbeg; k < q.kend; ++k) {
        const int s = it % S;
        if (!mbar_wait(&full[s], (it / S) & 1, g.status)) {
          *fail = 1;
          break;
        }
        tc_fence_after();
        const uint32_t sa = smem_u32(base + s * Lay::STAGE);
        const uint32_t sb = sa + Lay::A_BYTES;
        const uint64_t da = smem_desc<RB>(sa), db = smem_desc<RB>(sb);
#pragma unroll
        for (int kk = 0; kk < KSTEPS; ++kk)
          mma_bf16(d, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, (k > q.kbeg || kk > 0) ? 1u : 0u);
        mma_commit(&empty[s]);
        ++it;
      }
      if (*fail) break;
      mma_commit(&acc_full[buf]);
    }
    s_consumed = it;
    mma_commit(done);  // completes once every MMA issued above has finished
  } else if (warp >= 2) {
    // ---- epilogue
    const int quarter = warp & 3;
    const int row = quarter * 32 + lane;  // TMEM lane == tile row
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      const GemmTile q = decode_tile<BN>(g, t);
      if (q.kend <= q.kbeg) continue;
      const int buf = lt & 1;
      // the decision is warp-uniform (tcgen05.ld is a warp collective)
      const bool got = __all_sync(0xffffffffu, !*fail && mbar_wait(&acc_full[buf], (lt >> 1) & 1, g.status));
      if (!got) {
        *fail = 1;
        break;
      }
      tc_fence_after();
      const uint32_t taddr = tmem + (uint32_t)(buf * Lay::ACC_COLS) + ((uint32_t)(quarter * 32) << 16);
      if (g.mode == MODE_CONV) {
        const int py = q.y0 + row / g.TW, px = q.x0 + row % g.TW;
        const bool inrow = py < g.H && px < g.W;
        const long long pix = ((long long)q.n_img * g.H + py) * g.W + px;
        const bool vb = ((g.out_cstride | g.out_coff) & 7) == 0;
        const bool vf = ((g.out_cstride | g.out_coff) & 3) == 0;
        const bool vm = (g.mask_cstride & 7) == 0;
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
          float v[16];
          tmem_ld16(taddr + c, v);
          const int co = q.n0 + c;
          if (!inrow || co >= g.Cout) continue;
          const bool whole = co + 16 <= g.Cout;
          if (g.bias != nullptr) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += (co + j < g.Cout) ? __ldg(g.bias + co + j) : 0.f;
          }
          if (g.relu) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = v[j] < 0.f ? 0.f : v[j];
          }
          if (g.mask != nullptr) {
            const __nv_bfloat16* mp = g.mask + pix * g.mask_cstride + co;
            if (whole && vm) {
              const uint4 m0 = __ldg(reinterpret_cast<const uint4*>(mp));
              const uint4 m1 = __ldg(reinterpret_cast<const uint4*>(mp + 8));
              const __nv_bfloat16* mb0 = reinterpret_cast<const __nv_bfloat16*>(&m0);
              const __nv_bfloat16* mb1 = reinterpret_cast<const __nv_bfloat16*>(&m1);
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                v[j] = __bfloat162float(mb0[j]) > 0.f ? v[j] : 0.f;
                v[8 + j] = __bfloat162float(mb1[j]) > 0.f ? v[8 + j] : 0.f;
              }
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j)
                if (co + j < g.Cout) v[j] = __bfloat162float(mp[j]) > 0.f ? v[j] : 0.f;
            }
          }
          if (g.out_f32 != nullptr) {
            float* o = g.out_f32 + pix * g.out_cstride + g.out_coff + co;
            if (whole && vf) {
#pragma unroll
              for (int j = 0; j < 16; j += 4)
                *reinterpret_cast<float4*>(o + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j)
                if (co + j < g.Cout) o[j] = v[j];
            }
          }
          if (g.out_bf16 != nullptr) {
            __nv_bfloat16* o = g.out_bf16 + pix * g.out_cstride + g.out_coff + co;
            if (whole && vb) {
              st_bf16x8(o, v);
              st_bf16x8(o + 8, v + 8);
            } else {
#pragma unroll
              for (int j = 0; j < 16; ++j)
                if (co + j < g.Cout) o[j] = __float2bfloat16_rn(v[j]);
            }
          }
        }
      } else {
        // dW[co][ci][tap] += D[co][ci]   (the [cout][cin][3][3] layout)
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
          float v[16];
          tmem_ld16(taddr + c, v);
          const int co = q.m0 + row;
          if (co >= g.Cout) continue;
          float* o = g.out_f32 + ((long long)co * g.Cin + q.n0 + c) * 9 + q.tap;
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (q.n0 + c + j < g.Cin) atomicAdd(o + 9 * j, v[j]);
        }
      }
      // the buffer is free once every lane's tcgen05.ld has completed
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[buf]);
    }
  }
  __syncthreads();
  // ---- drain: every MMA issued, and the boxes issued but never consumed
  // (only after a failure), complete before the TMEM and the stages go
  if (threadIdx.x == 32) mbar_wait(done, 0, nullptr);
  if (threadIdx.x == 0 && *fail)
    for (int i = s_consumed; i < s_issued; ++i) mbar_wait(&full[i % S], (i / S) & 1, nullptr);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(Lay::TMEM_COLS)
                 : "memory");
  }
}

template <int BN, int RB>
cudaError_t launch_t(const CUtensorMap* maps, const GemmArgs& g0, dim3 grid, cudaStream_t s) {
  constexpr int S = (BN == 128 && RB == 128) ? 3 : 4;
  using Lay = GemmLayout<BN, RB, S>;
  auto kern = nn_gemm_kernel<BN, RB, S>;
  // The resident CTAs' accumulators must fit the SM's 512 TMEM columns
  // (a CTA beyond that would wait in tcgen05.alloc until a neighbour
  // exits): where shared memory alone would admit more CTAs, each CTA asks
  // for enough shared memory that only tm fit.
  static int per_sm = 0;
  static int smem = Lay::BYTES;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (per_sm == 0) {
    const int tm = 512 / Lay::TMEM_COLS;
    int sm_bytes = 0;
    cudaDeviceGetAttribute(&sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int pad = sm_bytes / (tm + 1) + 1;  // tm + 1 CTAs of this size no longer fit
    if (pad > smem) smem = pad;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    // residency from the kernel's own resources: registers (allocated per
    // warp in units of 256), static + dynamic shared memory (plus the 1 KB
    // the system reserves per CTA), TMEM columns
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, kern);
    if (e != cudaSuccess) return e;
    int regs_sm = 0;
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
    const int by_regs = warp_regs > 0 ? regs_sm / (warp_regs * 6) : 1;
    const int by_smem = sm_bytes / ((int)fa.sharedSizeBytes + smem + 1024);
    int nb = by_regs < by_smem ? by_regs : by_smem;
    if (nb < 1) nb = 1;
    per_sm = nb < tm ? nb : tm;
  }
  GemmArgs g = g0;
  g.gx = (int)grid.x;
  g.gy = (int)grid.y;
  g.gz = (int)grid.z;
  const long long ntiles = (long long)grid.x * grid.y * grid.z;
  if (ntiles <= 0) return cudaSuccess;
  const long long cap = (long long)per_sm * (sms > 0 ? sms : 152);
  const unsigned nblk = (unsigned)(ntiles < cap ? ntiles : cap);
  kern<<<nblk, 192, smem, s>>>(maps[0], maps[1], maps[2], maps[3], g);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gemm(int bn, int rb, const CUtensorMap* maps, const GemmArgs& g, dim3 grid, cudaStream_t s) {
  if (rb == 128) {
    switch (bn) {
      case 32: return launch_t<32, 128>(maps, g, grid, s);
      case 64: return launch_t<64, 128>(maps, g, grid, s);
      case 128: return launch_t<128, 128>(maps, g, grid, s);
    }
  } else if (rb == 64) {
    switch (bn) {
      case 32: return launch_t<32, 64>(maps, g, grid, s);
      case 64: return launch_t<64, 64>(maps, g, grid, s);
      case 128: return launch_t<128, 64>(maps, g, grid, s);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace nn
}  // namespace sgb
