// Boundary-saving adjoint of the acoustic HABC loop (acoustic_habc.py:79-221).
//
// The HABC step is linear in (U_n, U_{n-1}):
//   y       = 2 U_n - U_{n-1} + k L(U_n)                      (every cell)
//   out[p]  = (1 - b_p sum_s W_s(p)) y[p] + b_p sum_s W_s(p) one_s(p)
// where W_s(p) in {0, 1/2, 1} is side s's share of cell p after the mask
// precedence (top < bottom < left < right) and the 0.5/0.5 corner diagonals
// (acoustic_habc.py:167-202), and one_s(p) is the one-way extrapolation of
// side s along its inward normal d at depth k (acoustic_habc.py:79-101):
//   one = (2-lam-mu) U_n[p] + (lam+2mu) U_n[p+d] - mu U_n[p2]
//         + (lam-1) U_{n-1}[p] - lam U_{n-1}[p+d],
//   lam = 2 vp dt / h, mu = vp^2 dt^2 / h^2, p2 = p + 2d, or the line's edge
//   cell when k = hw - 1 (the reference's roll of the 51-deep slab).
// The reverse step gathers the transpose for every cell q:
//   La_j[q] = 2 wi(q) La1(q) + L(k wi La1)(q) - wi(q) La2(q)
//             + sum_s [one-way transposes of La1 and La2 along side s]
//             + receiver residuals,         wi = 1 - b sum_s W_s,
// with La1 = La_{j+1}, La2 = La_{j+2}.  Inside the undamped interior box
// the forward is the plain update, so the wavefield is reconstructed as in
// the PML adjoint (U_{j-2} = 2 U_{j-1} - (U_j - S w) + k L(U_{j-1})) and
// dJ/dvp += La_j (2k / vp) L(U_{j-1}) there; the ring of order/2 cells
// around the box comes from the forward's store.
//
// One kernel takes each reverse step (habc_bwd_tile_kernel, 8 x 128 tiles
// staged in shared memory), in two instantiations: tiles out of reach of
// every strip (wi = 1 over the whole stencil, no one-way line) and tiles
// near a strip (static shares from planes filled once per reverse loop,
// one-way transposes gathered from the staged La1 / La2).  The same
// equations carry the VTI (k Lx + kz Lz, vti_habc2.py), variable-density
// (C D(U), acoustic_rho_habc.py) and Born (the scattered field's adjoint
// against the background's reconstruction, acoustic_lsrtm_habc.py)
// gradients.
#include "sgb_common.cuh"
#include "acoustic_args.cuh"

namespace sgb {
namespace {

struct HabcW {
  float wi, wt, wb, wl, wr;  // interior share and the four sides' shares times b
};

// Side shares of cell (z, x): the same predicates as the forward kernel.
__device__ __forceinline__ HabcW habc_weights(int z, int x, int nz, int nx, int hw, bool mult, float b) {
  HabcW w{1.f, 0.f, 0.f, 0.f, 0.f};
  const int dT = z, dB = nz - 1 - z, dL = x, dR = nx - 1 - x;
  if (!(dT < hw || dB < hw || dL < hw || dR < hw)) return w;
  const bool top = !mult && dT < hw && dT <= dL && dT <= dR;
  const bool bot = dB < hw && dB <= dL && dB <= dR;
  const bool lft = dL < hw && ((mult && z < hw) || ((z >= hw || dL <= z) && (dB >= hw || dL <= dB)));
  const bool rgt = dR < hw && ((mult && z < hw) || ((z >= hw || dR <= z) && (dB >= hw || dR <= dB)));
  const bool tl = !mult && z < hw && x == z;
  const bool tr = !mult && z < hw && x == nx - hw + z;
  const bool bl = z >= nz - hw && x == z - (nz - hw);
  const bool br = z >= nz - hw && x == nx - hw + z - (nz - hw);
  float T = 0.f, B = 0.f, Lf = 0.f, Rt = 0.f;
  // later assignments win, as in the forward
  if (top) { T = 1.f; B = Lf = Rt = 0.f; }
  if (bot) { B = 1.f; T = Lf = Rt = 0.f; }
  if (lft) { Lf = 1.f; T = B = Rt = 0.f; }
  if (rgt) { Rt = 1.f; T = B = Lf = 0.f; }
  if (tl) { T = 0.5f; Lf = 0.5f; B = Rt = 0.f; }
  if (tr) { T = 0.5f; Rt = 0.5f; B = Lf = 0.f; }
  if (bl) { B = 0.5f; Lf = 0.5f; T = Rt = 0.f; }
  if (br) { B = 0.5f; Rt = 0.5f; T = Lf = 0.f; }
  const float sum = T + B + Lf + Rt;
  w.wi = 1.f - b * sum;
  w.wt = b * T;
  w.wb = b * B;
  w.wl = b * Lf;
  w.wr = b * Rt;
  return w;
}

struct HabcBwdArgs {
  int nz, nx, pitch, nshots, hw, multiple, R;
  // tile grid (ntx strips of HT_X columns, nzb bands of HT_Z rows) and the
  // block of far tiles, strips [fx0, fx1) x bands [fz0, fz1): the far
  // launch covers that block, the near launch the frame around it
  int ntx, nzb, fx0, fx1, fz0, fz1;
  long long sstride;
  const float* __restrict__ la1;   // La_{j+1}
  const float* __restrict__ la2;   // La_{j+2}
  float* __restrict__ lout;        // La_j
  const float* __restrict__ uj;    // U_j
  const float* __restrict__ ujm1;  // U_{j-1}
  float* __restrict__ uout;        // U_{j-2}, or null
  float* __restrict__ grad;        // [nshots][nz][pitch] += La_j k L(U_{j-1}) inside the box
  const float* __restrict__ k;     // vp^2 dt^2 / h^2 (VTI: the x coefficient plane)
  const float* __restrict__ kz;    // VTI: the z coefficient plane (update k Lx + kz Lz), else null
  float* __restrict__ grad2;       // VTI: [nshots][nz][pitch] += La_j Lz(U_{j-1}); grad gets La_j Lx(U_{j-1})
  // variable density: planes C, bx+, bx-, bz+, bz- (update C D(U)), and five
  // gradient fields [5][nshots][nz][pitch] (dJ/dC, dJ/dbx+, dJ/dbx-, dJ/dbz+, dJ/dbz-)
  const float* __restrict__ rho_c;
  float* __restrict__ grad_rho;
  const float* __restrict__ vp;
  const float* __restrict__ hb;    // blend weight b
  float lamf, muf;                 // 2 dt / h, dt^2 / h^2
  FdWeights w;
  Ring ring;
  const float* __restrict__ ring_in;  // ring of U_{j-2} [nshots][ring.size], or null (zeros)
  // sources of step j-1 (removed from U_j) and residuals of records j-1
  const int* __restrict__ src_ptr;
  const int* __restrict__ src_z;
  const int* __restrict__ src_x;
  const int* __restrict__ src_wrow;
  const float* __restrict__ wavelet;
  int nt, t_src;
  const int* __restrict__ rec_row_ptr;
  const int* __restrict__ rec_x;
  const int* __restrict__ rec_col;
  int nch;
  const float* __restrict__ resid;
  // [5][nz][pitch] static shares (wi, wt, wb, wl, wr) of every cell, or null
  const float* __restrict__ wpl;
};

__device__ __forceinline__ float ldz(const float* p, int z, int x, int nz, int nx, int pitch) {
  return (z >= 0 && z < nz && x >= 0 && x < nx) ? __ldg(p + (long long)z * pitch + x) : 0.f;
}

// One-way transpose of side s at cell q = (z, x): contributions of the
// strip cells p = q, q - d, q - 2d (and the wrap to the line's edge cell).
// depth(q) along s is dq; (sz, sx) is the inward step d.  USE1 / USE2 select
// the transposes of the U_n terms (applied to l1) and of the U_{n-1} terms
// (applied to l2).
template <bool USE1, bool USE2, class Args>
__device__ __forceinline__ float oneway_t(const Args& a, const float* l1, const float* l2, int z, int x, int dq,
                                          int sz, int sx, int side) {
  const int hw = a.hw;
  if (dq > hw) return 0.f;
  const bool mult = a.multiple != 0;
  float acc = 0.f;
  auto share = [&](int pz, int px) -> float {
    const long long o = (long long)pz * a.pitch + px;
    const HabcW w = habc_weights(pz, px, a.nz, a.nx, hw, mult, __ldg(a.hb + o));
    return side == 0 ? w.wt : side == 1 ? w.wb : side == 2 ? w.wl : w.wr;
  };
  auto coefs = [&](int pz, int px, float& lam, float& mu) {
    const float c = __ldg(a.vp + (long long)pz * a.pitch + px);
    lam = c * a.lamf;
    mu = c * c * a.muf;
  };
  // p = q (depth dq)
  if (dq < hw) {
    const float ws = share(z, x);
    if (ws != 0.f) {
      float lam, mu;
      coefs(z, x, lam, mu);
      const long long o = (long long)z * a.pitch + x;
      if (USE1) acc += ws * (2.f - lam - mu) * l1[o];
      if (USE2) acc += ws * (lam - 1.f) * l2[o];
    }
  }
  // p = q - d (depth dq - 1): U[p + d] and P[p + d] terms
  if (dq >= 1 && dq - 1 < hw) {
    const int pz = z - sz, px = x - sx;
    const float ws = share(pz, px);
    if (ws != 0.f) {
      float lam, mu;
      coefs(pz, px, lam, mu);
      const long long o = (long long)pz * a.pitch + px;
      if (USE1) acc += ws * (lam + 2.f * mu) * l1[o];
      if (USE2) acc -= ws * lam * l2[o];
    }
  }
  if (!USE1) return acc;
  // p = q - 2d (depth dq - 2, whose p2 is q when dq - 2 + 2 <= hw)
  if (dq >= 2 && dq <= hw) {
    const int pz = z - 2 * sz, px = x - 2 * sx;
    const float ws = share(pz, px);
    if (ws != 0.f) {
      float lam, mu;
      coefs(pz, px, lam, mu);
      acc -= ws * mu * l1[(long long)pz * a.pitch + px];
    }
  }
  // wrap: the depth hw-1 cell of this line reads the edge cell (depth 0)
  if (dq == 0) {
    const int pz = z + (hw - 1) * sz, px = x + (hw - 1) * sx;
    if (pz >= 0 && pz < a.nz && px >= 0 && px < a.nx) {
      const float ws = share(pz, px);
      if (ws != 0.f) {
        float lam, mu;
        coefs(pz, px, lam, mu);
        acc -= ws * mu * l1[(long long)pz * a.pitch + px];
      }
    }
  }
  return acc;
}

// Tiles of the reverse step: rows, columns, column halo (>= R).
constexpr int HT_Z = 8, HT_X = 128, HT_H = 4;


// ------------------------------------------------ single-step VJP ---
// The transpose of ONE step y = HABC(g (U - P) + P + I(U)) (I the
// equation's interior operator) for autograd of the per-step
// _time_step: gu = (dy/dU)^T G, gum = (dy/dP)^T G over the whole grid
// (strips included), the interior-operator parameter terms sum_b wi G dI/dtheta
// (plain: L(U), VTI: Lx(U) and Lz(U), variable density: D(U) and the four
// C-weighted one-cell differences), and the one-way terms' velocity
// derivative sum_b G sum_s ws d(one_s)/dvp.  With hw = 0 there is no blend
// (the reverse step of the boundary-saving path, acoustic_habc.py:223-245).
// Born (acoustic_lsrtm_habc.py:11-30): for the scattered field the source
// m k L(p) adds dJ/dm = sum_b wi G k L(p), its k term to the L plane and
// L(m k wi G) to dJ/dp.  One thread per cell loops over the shots, so the
// parameter sums need no atomics.
struct HabcVjpArgs {
  int nz, nx, pitch, nshots, hw, multiple;
  long long sstride;
  const float* __restrict__ u;
  const float* __restrict__ um;
  const float* __restrict__ gy;
  float* __restrict__ gu;
  float* __restrict__ gum;
  const float* __restrict__ g;
  const float* __restrict__ k;
  const float* __restrict__ kz;
  const float* __restrict__ rho_c;
  const float* __restrict__ vp;
  const float* __restrict__ hb;
  float lamf, muf;
  FdWeights w;
  float* __restrict__ gparam;  // [nplanes][nz][pitch]
  float* __restrict__ gc;      // [nz][pitch] or null
  const float* __restrict__ born_m;
  const float* __restrict__ born_u;
  float* __restrict__ born_gu;
  float* __restrict__ born_gm;
  float* __restrict__ wi_out;
};

template <int R, int EQ>
__global__ void __launch_bounds__(256) habc_step_vjp_kernel(const HabcVjpArgs a) {
  const long long cells = (long long)a.nz * a.nx;
  const long long pl = (long long)a.nz * a.pitch;
  const bool mult = a.multiple != 0;
  constexpr bool vti = EQ == 1;
  constexpr bool rho = EQ == 2 && R == 1;
  const bool born = EQ == 0 && a.born_m != nullptr;
  const float ch = 0.5f * a.w.c[0];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / a.nx), x = (int)(i - (long long)z * a.nx);
    const long long o = (long long)z * a.pitch + x;
    // every stencil neighbour in the grid and outside the strips: wi = 1
    const int far = a.hw + R;
    const bool interior = z >= (mult ? R : far) && a.nz - 1 - z >= far && x >= far && a.nx - 1 - x >= far;
    const HabcW wq = interior ? HabcW{1.f, 0.f, 0.f, 0.f, 0.f}
                              : habc_weights(z, x, a.nz, a.nx, a.hw, mult, __ldg(a.hb + o));
    auto wi_at = [&](int zz, int xx) -> float {
      return interior ? 1.f
                      : habc_weights(zz, xx, a.nz, a.nx, a.hw, mult, __ldg(a.hb + (long long)zz * a.pitch + xx)).wi;
    };
    const float gq = __ldg(a.g + o), kq = __ldg(a.k + o);
    const float kzq = vti ? __ldg(a.kz + o) : 0.f;
    const float mq = born ? __ldg(a.born_m + o) : 0.f;
    float pacc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    float cacc = 0.f, macc = 0.f;
    for (int b = 0; b < a.nshots; ++b) {
      const long long fb = (long long)b * a.sstride;
      const float* G = a.gy + fb;
      const float* U = a.u + fb;
      const float* P = a.um + fb;
      // weighted adjoint at a neighbour (0 off the grid), times a coefficient plane
      auto kwg = [&](int zz, int xx, const float* kp) -> float {
        if (zz < 0 || zz >= a.nz || xx < 0 || xx >= a.nx) return 0.f;
        const long long oo = (long long)zz * a.pitch + xx;
        return __ldg(kp + oo) * wi_at(zz, xx) * G[oo];
      };
      const float Gw = wq.wi * G[o];
      float tu;
      if (rho) {
        auto cw = [&](int zz, int xx, int q) -> float {
          if (zz < 0 || zz >= a.nz || xx < 0 || xx >= a.nx) return 0.f;
          const long long oo = (long long)zz * a.pitch + xx;
          return __ldg(a.rho_c + oo) * __ldg(a.rho_c + q * pl + oo) * wi_at(zz, xx) * G[oo];
        };
        const float sum = __ldg(a.rho_c + pl + o) + __ldg(a.rho_c + 2 * pl + o) + __ldg(a.rho_c + 3 * pl + o) +
                          __ldg(a.rho_c + 4 * pl + o);
        tu = gq * Gw - sum * __ldg(a.rho_c + o) * Gw + cw(z, x - 1, 1) + cw(z, x + 1, 2) + cw(z - 1, x, 3) +
             cw(z + 1, x, 4);
      } else if (vti) {
        float lap = ch * (kq + kzq) * Gw;
        for (int j = 1; j <= R; ++j)
          lap += a.w.c[j] * (kwg(z, x - j, a.k) + kwg(z, x + j, a.k) + kwg(z - j, x, a.kz) + kwg(z + j, x, a.kz));
        tu = gq * Gw + lap;
      } else {
        float lap = a.w.c[0] * kq * Gw;
        for (int j = 1; j <= R; ++j)
          lap += a.w.c[j] * (kwg(z - j, x, a.k) + kwg(z + j, x, a.k) + kwg(z, x - j, a.k) + kwg(z, x + j, a.k));
        tu = gq * Gw + lap;
      }
      float tum = (1.f - gq) * Gw;
      if (!interior && a.hw > 0) {
        tu += oneway_t<true, false>(a, G, nullptr, z, x, z, 1, 0, 0);
        tu += oneway_t<true, false>(a, G, nullptr, z, x, a.nz - 1 - z, -1, 0, 1);
        tu += oneway_t<true, false>(a, G, nullptr, z, x, x, 0, 1, 2);
        tu += oneway_t<true, false>(a, G, nullptr, z, x, a.nx - 1 - x, 0, -1, 3);
        tum += oneway_t<false, true>(a, nullptr, G, z, x, z, 1, 0, 0);
        tum += oneway_t<false, true>(a, nullptr, G, z, x, a.nz - 1 - z, -1, 0, 1);
        tum += oneway_t<false, true>(a, nullptr, G, z, x, x, 0, 1, 2);
        tum += oneway_t<false, true>(a, nullptr, G, z, x, a.nx - 1 - x, 0, -1, 3);
      }
      a.gu[fb + o] = tu;
      a.gum[fb + o] = tum;
      // interior-operator parameter terms (each cell's own coefficients)
      if (rho) {
        const float u0 = U[o];
        const float dxp = ldz(U, z, x + 1, a.nz, a.nx, a.pitch) - u0, dxn = u0 - ldz(U, z, x - 1, a.nz, a.nx, a.pitch);
        const float dzp = ldz(U, z + 1, x, a.nz, a.nx, a.pitch) - u0, dzn = u0 - ldz(U, z - 1, x, a.nz, a.nx, a.pitch);
        const float bxp = __ldg(a.rho_c + pl + o), bxn = __ldg(a.rho_c + 2 * pl + o);
        const float bzp = __ldg(a.rho_c + 3 * pl + o), bzn = __ldg(a.rho_c + 4 * pl + o);
        const float C = __ldg(a.rho_c + o);
        pacc[0] += Gw * (bxp * dxp - bxn * dxn + bzp * dzp - bzn * dzn);
        pacc[1] += Gw * C * dxp;
        pacc[2] -= Gw * C * dxn;
        pacc[3] += Gw * C * dzp;
        pacc[4] -= Gw * C * dzn;
      } else if (vti) {
        float Lx = ch * U[o], Lz = ch * U[o];
        for (int j = 1; j <= R; ++j) {
          Lx += a.w.c[j] * (ldz(U, z, x - j, a.nz, a.nx, a.pitch) + ldz(U, z, x + j, a.nz, a.nx, a.pitch));
          Lz += a.w.c[j] * (ldz(U, z - j, x, a.nz, a.nx, a.pitch) + ldz(U, z + j, x, a.nz, a.nx, a.pitch));
        }
        pacc[0] += Gw * Lx;
        pacc[1] += Gw * Lz;
      } else {
        float L = a.w.c[0] * U[o];
        for (int j = 1; j <= R; ++j)
          L += a.w.c[j] * (ldz(U, z - j, x, a.nz, a.nx, a.pitch) + ldz(U, z + j, x, a.nz, a.nx, a.pitch) +
                           ldz(U, z, x - j, a.nz, a.nx, a.pitch) + ldz(U, z, x + j, a.nz, a.nx, a.pitch));
        pacc[0] += Gw * L;
      }
      if (born) {  // source m k L(p): its k and m terms, and L(m k wi G) into dJ/dp
        const float* Pb = a.born_u + fb;
        float Lp = a.w.c[0] * Pb[o];
        float lg = a.w.c[0] * mq * kq * Gw;
        for (int j = 1; j <= R; ++j) {
          Lp += a.w.c[j] * (ldz(Pb, z - j, x, a.nz, a.nx, a.pitch) + ldz(Pb, z + j, x, a.nz, a.nx, a.pitch) +
                            ldz(Pb, z, x - j, a.nz, a.nx, a.pitch) + ldz(Pb, z, x + j, a.nz, a.nx, a.pitch));
          lg += a.w.c[j] * (kwg(z - j, x, a.born_m) * ldz(a.k, z - j, x, a.nz, a.nx, a.pitch) +
                            kwg(z + j, x, a.born_m) * ldz(a.k, z + j, x, a.nz, a.nx, a.pitch) +
                            kwg(z, x - j, a.born_m) * ldz(a.k, z, x - j, a.nz, a.nx, a.pitch) +
                            kwg(z, x + j, a.born_m) * ldz(a.k, z, x + j, a.nz, a.nx, a.pitch));
        }
        pacc[0] += Gw * mq * Lp;
        macc += Gw * kq * Lp;
        a.born_gu[fb + o] = lg;
      }
      // velocity derivative of the one-way extrapolations (lam = c lamf, mu = c^2 muf)
      if (!interior && a.hw > 0 && a.gc != nullptr) {
        const float c = __ldg(a.vp + o);
        const float dl = a.lamf, dm = 2.f * c * a.muf;
        auto done = [&](int dq, int sz, int sx, int ze, int xe) -> float {
          const long long d1 = (long long)sz * a.pitch + sx;
          const float U2 = (dq + 2 <= a.hw) ? U[o + 2 * d1] : U[(long long)ze * a.pitch + xe];
          return (-dl - dm) * U[o] + (dl + 2.f * dm) * U[o + d1] - dm * U2 + dl * P[o] - dl * P[o + d1];
        };
        float s = 0.f;
        if (wq.wt != 0.f) s += wq.wt * done(z, 1, 0, 0, x);
        if (wq.wb != 0.f) s += wq.wb * done(a.nz - 1 - z, -1, 0, a.nz - 1, x);
        if (wq.wl != 0.f) s += wq.wl * done(x, 0, 1, z, 0);
        if (wq.wr != 0.f) s += wq.wr * done(a.nx - 1 - x, 0, -1, z, a.nx - 1);
        cacc += G[o] * s;
      }
    }
    const int np = rho ? 5 : (vti ? 2 : 1);
    for (int q = 0; q < np; ++q) a.gparam[q * pl + o] = pacc[q];
    if (a.gc != nullptr) a.gc[o] = cacc;
    if (born) a.born_gm[o] = macc;
    if (a.wi_out != nullptr) a.wi_out[o] = wq.wi;
  }
}


// --------------------------------------------------- all-cell tiles ---
// The reverse step of every HABC equation, tile 8 x 128 with block (32, 8)
// (lane: four columns).  EQ 0 (plain, Born): La_j = 2 wi La1 + L(k wi La1)
// - wi La2; EQ 1 (VTI): x neighbours by kx, z neighbours by kz; EQ 2
// (variable density, R = 1): the transpose of C D, i.e. each neighbour's
// C wi La1 times the buoyancy of the half point between, from shared-memory
// tiles of (k or C) wi La1 and U_{j-1}; tiles within reach of a strip also stage La1 and La2
// (two-row halo) and add the one-way transposes of the four sides, with each
// cell's interior and side shares read from the five planes that
// habc_shares_kernel fills once per reverse loop; then the receiver
// residuals, the gradient term and the reconstruction inside the box, the
// saved ring (or 0) outside it.
template <int R, int EQ, bool NEAR>
__device__ __forceinline__ void habc_bwd_tile(const HabcBwdArgs& a) {
  constexpr bool VTI = EQ == 1, RHO = EQ == 2;
  static_assert(!RHO || R == 1, "variable density is second order");
  // row halo: the stencil's R, and 2 for the one-way lines (q - d, q - 2d)
  constexpr int HR = R < 2 ? 2 : R;
  constexpr int ROWS = HT_Z + 2 * HR, W = HT_X + 2 * HT_H;
  __shared__ __align__(16) float s_kl[ROWS][W];             // k wi La1 (VTI: kx wi La1; density: C wi La1)
  __shared__ __align__(16) float s_kzl[VTI ? ROWS : 1][W];  // VTI: kz wi La1
  __shared__ __align__(16) float s_u[ROWS][W];
  __shared__ __align__(16) float s_l1[NEAR ? ROWS : 1][W];  // La1 and La2 (tiles near a strip only)
  __shared__ __align__(16) float s_l2[NEAR ? ROWS : 1][W];
  const int b = blockIdx.z;
  int strip, band;
  if constexpr (!NEAR) {
    strip = a.fx0 + (int)blockIdx.x;
    band = a.fz0 + (int)blockIdx.y;
  } else {  // the frame: the bands above the far block, the strips beside it, the bands below
    int i = blockIdx.x;
    const int top = a.fz0 * a.ntx, nside = a.ntx - (a.fx1 - a.fx0), mid = (a.fz1 - a.fz0) * nside;
    if (i < top) {
      band = i / a.ntx;
      strip = i - band * a.ntx;
    } else if (i - top < mid) {
      i -= top;
      band = a.fz0 + i / nside;
      const int j = i - (i / nside) * nside;
      strip = j < a.fx0 ? j : a.fx1 + (j - a.fx0);
    } else {
      i -= top + mid;
      band = a.fz1 + i / a.ntx;
      strip = i - (i / a.ntx) * a.ntx;
    }
  }
  const int z0 = band * HT_Z, x0 = strip * HT_X;
  const long long fb = (long long)b * a.sstride;
  const float* l1 = a.la1 + fb;
  const float* u1 = a.ujm1 + fb;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int hw = a.hw;
  const bool mult = a.multiple != 0;
  const long long pl = (long long)a.nz * a.pitch;
  const float* __restrict__ kp = RHO ? a.rho_c : a.k;  // the plane that weights La1
  // does any cell of the tile or its halo have an interior share below 1, or
  // lie within reach of a one-way line (depth <= hw)?
  const bool near = hw > 0 && ((!mult && z0 - HR <= hw) || z0 + HT_Z + HR >= a.nz - 1 - hw ||
                                x0 - HT_H <= hw || x0 + HT_X + HT_H >= a.nx - 1 - hw);
  // two launches share the grid: the NEAR instantiation takes the tiles
  // within reach of a strip, the other the rest (with none of the strip code)
  if (near != NEAR) return;
  // interior shares of the four cells (z, x .. x+3), x a multiple of 4
  auto wi4_at = [&](int z, int x) -> float4 {
    if (!near) return make_float4(1.f, 1.f, 1.f, 1.f);
    const long long oo = (long long)z * a.pitch + x;
    if (a.wpl != nullptr) return __ldg(reinterpret_cast<const float4*>(a.wpl + oo));
    float4 r;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const float bb = x + m < a.nx ? __ldg(a.hb + oo + m) : 0.f;  // b = 0: no side share, wi = 1
      set_comp(r, m, bb == 0.f ? 1.f : habc_weights(z, x + m, a.nz, a.nx, hw, mult, bb).wi);
    }
    return r;
  };
  // stage (k or C) wi La1, U_{j-1} and, near a strip, La1 and La2 with their
  // halo.  Far tiles (and variable density) issue the loads of all of a
  // thread's groups first, then the point loads of its own four cells, and
  // only then write shared memory, so that one memory latency covers them
  // all; near tiles, issue-bound and short of registers, stage group by group.
  constexpr bool PRE = !NEAR || RHO;
  constexpr int NST = ROWS * (W / 4), NIT = (NST + 255) / 256;
  const float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f);
  struct Grp {
    float4 k, l, q, v, m, w;
  };
  auto stage_load = [&](int c, Grp& g) {
    const int rr_ = c / (W / 4), cc = c - rr_ * (W / 4);
    const int zs = z0 - HR + rr_, xs = x0 - HT_H + 4 * cc;
    g.k = g.l = g.q = g.v = g.m = f0;
    g.w = make_float4(1.f, 1.f, 1.f, 1.f);
    if (c < NST && zs >= 0 && zs < a.nz && xs >= 0 && xs < a.nx) {
      const long long os = (long long)zs * a.pitch + xs;
      g.k = __ldg(reinterpret_cast<const float4*>(kp + os));
      g.l = *reinterpret_cast<const float4*>(l1 + os);
      if (VTI) g.q = __ldg(reinterpret_cast<const float4*>(a.kz + os));
      g.v = *reinterpret_cast<const float4*>(u1 + os);
      if (NEAR) g.m = *reinterpret_cast<const float4*>(a.la2 + fb + os);
      if (NEAR) g.w = wi4_at(zs, xs);
    }
  };
  auto stage_store = [&](int c, Grp& g) {
    const int rr_ = c / (W / 4), cc = c - rr_ * (W / 4);
    const int xs = x0 - HT_H + 4 * cc;
    float kl[4] = {0.f, 0.f, 0.f, 0.f}, kzl[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (xs + m < a.nx) {  // columns beyond the grid stay 0
        const float w = comp(g.w, m);
        kl[m] = comp(g.k, m) * w * comp(g.l, m);
        if (VTI) kzl[m] = comp(g.q, m) * w * comp(g.l, m);
      } else {
        set_comp(g.v, m, 0.f);
        set_comp(g.l, m, 0.f);
        set_comp(g.m, m, 0.f);
      }
    }
    *reinterpret_cast<float4*>(&s_kl[rr_][4 * cc]) = make_float4(kl[0], kl[1], kl[2], kl[3]);
    if (VTI) *reinterpret_cast<float4*>(&s_kzl[rr_][4 * cc]) = make_float4(kzl[0], kzl[1], kzl[2], kzl[3]);
    *reinterpret_cast<float4*>(&s_u[rr_][4 * cc]) = g.v;
    if constexpr (NEAR) {
      *reinterpret_cast<float4*>(&s_l1[rr_][4 * cc]) = g.l;
      *reinterpret_cast<float4*>(&s_l2[rr_][4 * cc]) = g.m;
    }
  };
  const int z = z0 + threadIdx.y, x = x0 + 4 * threadIdx.x;
  const bool cell_in = z < a.nz && x < a.nx;
  const int rr = HR + threadIdx.y, cx = HT_H + 4 * threadIdx.x;
  const long long o = (long long)z * a.pitch + x;
  const bool row_in = z >= a.ring.iz0 && z < a.ring.iz1;
  const bool box4 = row_in && x >= a.ring.ix0 && x + 3 < a.ring.ix1;  // all four cells inside the box
  float4 k4 = f0, kz4 = f0, l2g = f0, l1g = f0, uj4 = f0;
  auto point_loads = [&]() {
    if (!cell_in) return;
    k4 = __ldg(reinterpret_cast<const float4*>(kp + o));
    if (VTI) kz4 = __ldg(reinterpret_cast<const float4*>(a.kz + o));
    if (!NEAR) {
      l2g = *reinterpret_cast<const float4*>(a.la2 + fb + o);
      l1g = *reinterpret_cast<const float4*>(l1 + o);
    }
  };
  // U_j of the four cells (reconstruction)
  auto tail_loads = [&]() {
    if (!cell_in) return;
    if (a.uout != nullptr && row_in) uj4 = *reinterpret_cast<const float4*>(a.uj + fb + o);
  };
  if constexpr (PRE) {
    Grp g[NIT];
#pragma unroll
    for (int it = 0; it < NIT; ++it) stage_load(tid + 256 * it, g[it]);
    point_loads();
    tail_loads();
#pragma unroll
    for (int it = 0; it < NIT; ++it)
      if (tid + 256 * it < NST) stage_store(tid + 256 * it, g[it]);
  } else {
    for (int c = tid; c < NST; c += 256) {
      Grp g;
      stage_load(c, g);
      stage_store(c, g);
    }
  }
  __syncthreads();
  if (!cell_in) return;
  if constexpr (!PRE) point_loads();
  if (!VTI) kz4 = k4;
  // La2 and La1 of the four cells (staged in near tiles)
  const float4 l2v = NEAR ? *reinterpret_cast<const float4*>(&s_l2[rr][cx]) : l2g;
  const float4 l1c = NEAR ? *reinterpret_cast<const float4*>(&s_l1[rr][cx]) : l1g;
  // variable density: the four half-point buoyancies of the cells (bx+, bx-,
  // bz+, bz-), bz+ of the row above, bz- of the row below, bx+ of the
  // column left of the group and bx- of the column right of it
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 bxp = z4, bxn = z4, bzp = z4, bzn = z4, bzpU = z4, bznD = z4;
  float bxpL = 0.f, bxnR = 0.f;
  if constexpr (RHO) {
    bxp = __ldg(reinterpret_cast<const float4*>(a.rho_c + pl + o));
    bxn = __ldg(reinterpret_cast<const float4*>(a.rho_c + 2 * pl + o));
    bzp = __ldg(reinterpret_cast<const float4*>(a.rho_c + 3 * pl + o));
    bzn = __ldg(reinterpret_cast<const float4*>(a.rho_c + 4 * pl + o));
    if (z > 0) bzpU = __ldg(reinterpret_cast<const float4*>(a.rho_c + 3 * pl + o - a.pitch));
    if (z + 1 < a.nz) bznD = __ldg(reinterpret_cast<const float4*>(a.rho_c + 4 * pl + o + a.pitch));
    if (x > 0) bxpL = __ldg(a.rho_c + pl + o - 1);
    if (x + 4 < a.nx) bxnR = __ldg(a.rho_c + 2 * pl + o + 4);
  }
  // one-way transposes of side `sd` at cell (z, xm) of local column cxm:
  // strip cells p = q, q - d, q - 2d (staged La1 / La2) and the wrap of the
  // line's depth hw-1 cell into its edge cell (global)
  auto share = [&](int sd, int pz, int px) -> float {
    const long long oo = (long long)pz * a.pitch + px;
    if (a.wpl != nullptr) return __ldg(a.wpl + (1 + sd) * pl + oo);
    const float bb = __ldg(a.hb + oo);
    if (bb == 0.f) return 0.f;
    const HabcW w = habc_weights(pz, px, a.nz, a.nx, hw, mult, bb);
    return sd == 0 ? w.wt : sd == 1 ? w.wb : sd == 2 ? w.wl : w.wr;
  };
  auto oneway = [&](int sd, int dq, int sz, int sx, int xm, int cxm) -> float {
    if (dq > hw) return 0.f;
    float acc = 0.f;
    if (dq < hw) {
      const float ws = share(sd, z, xm);
      if (ws != 0.f) {
        const float c = __ldg(a.vp + (long long)z * a.pitch + xm);
        const float lam = c * a.lamf, mu = c * c * a.muf;
        acc += ws * ((2.f - lam - mu) * s_l1[rr][cxm] + (lam - 1.f) * s_l2[rr][cxm]);
      }
    }
    if (dq >= 1) {
      const int pz = z - sz, px = xm - sx;
      const float ws = share(sd, pz, px);
      if (ws != 0.f) {
        const float c = __ldg(a.vp + (long long)pz * a.pitch + px);
        const float lam = c * a.lamf, mu = c * c * a.muf;
        acc += ws * ((lam + 2.f * mu) * s_l1[rr - sz][cxm - sx] - lam * s_l2[rr - sz][cxm - sx]);
      }
    }
    if (dq >= 2) {
      const int pz = z - 2 * sz, px = xm - 2 * sx;
      const float ws = share(sd, pz, px);
      if (ws != 0.f) {
        const float c = __ldg(a.vp + (long long)pz * a.pitch + px);
        acc -= ws * c * c * a.muf * s_l1[rr - 2 * sz][cxm - 2 * sx];
      }
    }
    if (dq == 0) {
      const int pz = z + (hw - 1) * sz, px = xm + (hw - 1) * sx;
      if (pz >= 0 && pz < a.nz && px >= 0 && px < a.nx) {
        const float ws = share(sd, pz, px);
        if (ws != 0.f) {
          const long long oo = (long long)pz * a.pitch + px;
          const float c = __ldg(a.vp + oo);
          acc -= ws * c * c * a.muf * l1[oo];
        }
      }
    }
    return acc;
  };
  // top / bottom sides: the four cells share their depth dq, so the strip
  // cells p = q, q - d, q - 2d (and the wrap) are rows of four
  auto share4 = [&](int sd, int pz) -> float4 {
    const long long oo = (long long)pz * a.pitch + x;
    if (a.wpl != nullptr) return __ldg(reinterpret_cast<const float4*>(a.wpl + (1 + sd) * pl + oo));
    float4 r;
#pragma unroll
    for (int m = 0; m < 4; ++m) set_comp(r, m, x + m < a.nx ? share(sd, pz, x + m) : 0.f);
    return r;
  };
  auto oneway_rows = [&](int sd, int dq, int sz, float4& acc) {
    auto coefs = [&](int pz, float4& lam, float4& mu) {
      const float4 c = __ldg(reinterpret_cast<const float4*>(a.vp + (long long)pz * a.pitch + x));
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        set_comp(lam, m, comp(c, m) * a.lamf);
        set_comp(mu, m, comp(c, m) * comp(c, m) * a.muf);
      }
    };
    float4 lam, mu;
    if (dq < hw) {
      const float4 ws = share4(sd, z);
      coefs(z, lam, mu);
#pragma unroll
      for (int m = 0; m < 4; ++m)
        set_comp(acc, m, comp(acc, m) + comp(ws, m) * ((2.f - comp(lam, m) - comp(mu, m)) * s_l1[rr][cx + m] +
                                                       (comp(lam, m) - 1.f) * s_l2[rr][cx + m]));
    }
    if (dq >= 1) {
      const float4 ws = share4(sd, z - sz);
      coefs(z - sz, lam, mu);
#pragma unroll
      for (int m = 0; m < 4; ++m)
        set_comp(acc, m, comp(acc, m) + comp(ws, m) * ((comp(lam, m) + 2.f * comp(mu, m)) * s_l1[rr - sz][cx + m] -
                                                       comp(lam, m) * s_l2[rr - sz][cx + m]));
    }
    if (dq >= 2) {
      const float4 ws = share4(sd, z - 2 * sz);
      coefs(z - 2 * sz, lam, mu);
#pragma unroll
      for (int m = 0; m < 4; ++m)
        set_comp(acc, m, comp(acc, m) - comp(ws, m) * comp(mu, m) * s_l1[rr - 2 * sz][cx + m]);
    }
    if (dq == 0) {
      const int pz = z + (hw - 1) * sz;
      if (pz >= 0 && pz < a.nz) {
        const float4 ws = share4(sd, pz);
        coefs(pz, lam, mu);
        const float4 lw = *reinterpret_cast<const float4*>(l1 + (long long)pz * a.pitch + x);
#pragma unroll
        for (int m = 0; m < 4; ++m) set_comp(acc, m, comp(acc, m) - comp(ws, m) * comp(mu, m) * comp(lw, m));
      }
    }
  };
  // the one-way sums of the four cells: rows of four for the top and bottom
  // sides; cell by cell (one rolled copy of the code) for the left and right
  // sides, in the lanes within their reach only
  float4 ow4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (NEAR) {
    if (!mult && z <= hw) oneway_rows(0, z, 1, ow4);
    if (a.nz - 1 - z <= hw) oneway_rows(1, a.nz - 1 - z, -1, ow4);
    if (x <= hw || x + 3 >= a.nx - 1 - hw) {
#pragma unroll 1
      for (int t = 0; t < 8; ++t) {
        const int m = t >> 1, sd = 2 + (t & 1);
        const int xm = x + m;
        if (xm >= a.nx) continue;
        const int dq = sd == 2 ? xm : a.nx - 1 - xm;
        if (dq > hw) continue;
        set_comp(ow4, m, comp(ow4, m) + oneway(sd, dq, 0, sd == 2 ? 1 : -1, xm, cx + m));
      }
    }
  }
  const float4 wq4 = wi4_at(z, x);
  const float ch = 0.5f * a.w.c[0];
  float v[4], L[4], Lz[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int xm = x + m;
    const float wq = (xm < a.nx) ? comp(wq4, m) : 0.f;
    const float ow = NEAR ? comp(ow4, m) : 0.f;
    float lap, lu, luz = 0.f;
    if (RHO) {
      const float bl = m == 0 ? bxpL : comp(bxp, m - 1);
      const float br = m == 3 ? bxnR : comp(bxn, m + 1);
      lap = -(comp(bxp, m) + comp(bxn, m) + comp(bzp, m) + comp(bzn, m)) * s_kl[rr][cx + m] +
            bl * s_kl[rr][cx + m - 1] + br * s_kl[rr][cx + m + 1] + comp(bzpU, m) * s_kl[rr - 1][cx + m] +
            comp(bznD, m) * s_kl[rr + 1][cx + m];
      // D(U_{j-1}) of the cell's own half points
      const float u0 = s_u[rr][cx + m];
      const float dxp = s_u[rr][cx + m + 1] - u0, dxn = u0 - s_u[rr][cx + m - 1];
      const float dzp = s_u[rr + 1][cx + m] - u0, dzn = u0 - s_u[rr - 1][cx + m];
      lu = comp(bxp, m) * dxp - comp(bxn, m) * dxn + comp(bzp, m) * dzp - comp(bzn, m) * dzn;
      luz = 0.f;
    } else if (VTI) {
      float lx = ch * s_kl[rr][cx + m], lz = ch * s_kzl[rr][cx + m];
      float ux = ch * s_u[rr][cx + m], uz = ch * s_u[rr][cx + m];
#pragma unroll
      for (int j = 1; j <= R; ++j) {
        lx += a.w.c[j] * (s_kl[rr][cx + m - j] + s_kl[rr][cx + m + j]);
        lz += a.w.c[j] * (s_kzl[rr - j][cx + m] + s_kzl[rr + j][cx + m]);
        ux += a.w.c[j] * (s_u[rr][cx + m - j] + s_u[rr][cx + m + j]);
        uz += a.w.c[j] * (s_u[rr - j][cx + m] + s_u[rr + j][cx + m]);
      }
      lap = lx + lz;
      lu = ux;
      luz = uz;
    } else {
      lap = a.w.c[0] * s_kl[rr][cx + m];
      lu = a.w.c[0] * s_u[rr][cx + m];
#pragma unroll
      for (int j = 1; j <= R; ++j) {
        lap += a.w.c[j] * (s_kl[rr - j][cx + m] + s_kl[rr + j][cx + m] + s_kl[rr][cx + m - j] + s_kl[rr][cx + m + j]);
        lu += a.w.c[j] * (s_u[rr - j][cx + m] + s_u[rr + j][cx + m] + s_u[rr][cx + m - j] + s_u[rr][cx + m + j]);
      }
    }
    v[m] = (xm < a.nx) ? 2.f * wq * comp(l1c, m) + lap - wq * comp(l2v, m) + ow : 0.f;
    L[m] = lu;
    Lz[m] = luz;
  }
  // residuals of the records of step j-1 in this row
  if (a.resid != nullptr) {
    const int* rp = a.rec_row_ptr + (long long)b * a.nz;
    int lo = rp[z], hi = rp[z + 1];
    const int end = hi;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (a.rec_x[mid] < x) lo = mid + 1; else hi = mid;
    }
    for (int q = lo; q < end && a.rec_x[q] < x + 4; ++q) {
      const int dx = a.rec_x[q] - x;
      const float rv = a.resid[(long long)a.rec_col[q] * a.nch];
#pragma unroll
      for (int m = 0; m < 4; ++m)
        if (dx == m) v[m] += rv;
    }
  }
  *reinterpret_cast<float4*>(a.lout + fb + o) = make_float4(v[0], v[1], v[2], v[3]);
  // gradient and reconstruction inside the box; the saved ring (or 0) outside
  if constexpr (!PRE) tail_loads();
  float uo[4] = {0.f, 0.f, 0.f, 0.f};
  float ujv[4] = {0.f, 0.f, 0.f, 0.f};
  if (a.uout != nullptr && row_in) {
    ujv[0] = uj4.x; ujv[1] = uj4.y; ujv[2] = uj4.z; ujv[3] = uj4.w;
    if (a.src_ptr != nullptr) {
      for (int q = a.src_ptr[b]; q < a.src_ptr[b + 1]; ++q) {
        const int dx = a.src_x[q] - x;
        if (a.src_z[q] == z && dx >= 0 && dx < 4) {
          const float wv = a.wavelet[(long long)a.src_wrow[q] * a.nt + a.t_src];
#pragma unroll
          for (int m = 0; m < 4; ++m)
            if (dx == m) ujv[m] -= wv;
        }
      }
    }
  }
  // variable density: the five gradient terms of cell m (dJ/dC and the
  // four buoyancies) from La_j and the differences of U_{j-1}
  const long long fs = (long long)a.nshots * a.sstride;  // one density gradient field
  auto rho_terms = [&](int m, float t[5]) {
    const float u0 = s_u[rr][cx + m], vC = v[m] * comp(k4, m);
    t[0] = v[m] * L[m];
    t[1] = vC * (s_u[rr][cx + m + 1] - u0);
    t[2] = -vC * (u0 - s_u[rr][cx + m - 1]);
    t[3] = vC * (s_u[rr + 1][cx + m] - u0);
    t[4] = -vC * (u0 - s_u[rr - 1][cx + m]);
  };
  // gradient terms: every shot adds into plane 0 of its gradient field(s)
  // (16-byte reductions in L2; the shot reduction reads that plane)
  if (box4) {
    // all four columns inside the box: vector gradient update and reconstruction
    if constexpr (RHO) {
      float t[4][5];
#pragma unroll
      for (int m = 0; m < 4; ++m) rho_terms(m, t[m]);
#pragma unroll
      for (int q = 0; q < 5; ++q) red_add4(a.grad_rho + q * fs + o, make_float4(t[0][q], t[1][q], t[2][q], t[3][q]));
    } else if (VTI) {
      red_add4(a.grad + o, make_float4(v[0] * L[0], v[1] * L[1], v[2] * L[2], v[3] * L[3]));
      red_add4(a.grad2 + o, make_float4(v[0] * Lz[0], v[1] * Lz[1], v[2] * Lz[2], v[3] * Lz[3]));
    } else {
      red_add4(a.grad + o, make_float4(v[0] * k4.x * L[0], v[1] * k4.y * L[1], v[2] * k4.z * L[2], v[3] * k4.w * L[3]));
    }
    if (a.uout != nullptr) {
#pragma unroll
      for (int m = 0; m < 4; ++m)
        uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + comp(k4, m) * L[m] + (VTI ? comp(kz4, m) * Lz[m] : 0.f);
      *reinterpret_cast<float4*>(a.uout + fb + o) = make_float4(uo[0], uo[1], uo[2], uo[3]);
    }
    return;
  }
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int xm = x + m;
    if (xm >= a.nx) break;
    const long long om = o + m;
    if (row_in && xm >= a.ring.ix0 && xm < a.ring.ix1) {
      const float kk = comp(k4, m);
      if (RHO) {
        float t[5];
        rho_terms(m, t);
#pragma unroll
        for (int q = 0; q < 5; ++q) atomicAdd(a.grad_rho + q * fs + om, t[q]);
        uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + kk * L[m];
      } else if (VTI) {
        atomicAdd(a.grad + om, v[m] * L[m]);
        atomicAdd(a.grad2 + om, v[m] * Lz[m]);
        uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + kk * L[m] + comp(kz4, m) * Lz[m];
      } else {
        atomicAdd(a.grad + om, v[m] * kk * L[m]);
        uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + kk * L[m];
      }
    } else {
      if constexpr (RHO) {
        // the box's one-cell rim: the half-point buoyancy terms that reach
        // into the box (their U values are the box's and the saved ring's),
        // so that dJ/drho is complete at the box's edge cells
        const bool xr = a.ring.inside(z, xm + 1), xl = a.ring.inside(z, xm - 1);
        const bool zd = a.ring.inside(z + 1, xm), zu = a.ring.inside(z - 1, xm);
        if (xr || xl || zd || zu) {
          float t[5];
          rho_terms(m, t);
          if (xr) atomicAdd(a.grad_rho + fs + om, t[1]);
          if (xl) atomicAdd(a.grad_rho + 2 * fs + om, t[2]);
          if (zd) atomicAdd(a.grad_rho + 3 * fs + om, t[3]);
          if (zu) atomicAdd(a.grad_rho + 4 * fs + om, t[4]);
        }
      }
      if (a.uout != nullptr) {
        const int ri = a.ring.index(z, xm);
        uo[m] = (ri >= 0 && a.ring_in != nullptr) ? a.ring_in[(long long)b * a.ring.size + ri] : 0.f;
      }
    }
  }
  if (a.uout != nullptr) *reinterpret_cast<float4*>(a.uout + fb + o) = make_float4(uo[0], uo[1], uo[2], uo[3]);
}

// The plain / Born equation's kernel is left to the compiler's register
// choice; the VTI and variable-density ones are held to the CTAs per SM
// (eight warps each) that their registers allowed before the tile index
// came from the far block or the frame: near tiles four (variable density
// two), far tiles three (VTI of order 6 and 8 two).
template <int R, int EQ, bool NEAR>
constexpr int habc_bwd_min_blocks() {
  if (NEAR) return EQ == 2 ? 2 : 4;
  if (EQ == 2) return 3;
  return R <= 2 ? 3 : 2;
}
template <int R, int EQ, bool NEAR>
__global__ void __launch_bounds__(256) habc_bwd_tile_kernel(const HabcBwdArgs a) {
  habc_bwd_tile<R, EQ, NEAR>(a);
}
template <int R, int EQ, bool NEAR>
__global__ void __launch_bounds__(256, habc_bwd_min_blocks<R, EQ, NEAR>()) habc_bwd_tile_kernel_held(
    const HabcBwdArgs a) {
  habc_bwd_tile<R, EQ, NEAR>(a);
}


// The static shares of every cell: wi and the four sides' b * share.
__global__ void habc_shares_kernel(int nz, int nx, int pitch, int hw, int mult, const float* __restrict__ hb,
                                   float* __restrict__ out) {
  const long long pl = (long long)nz * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < pl; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / pitch), x = (int)(i - (long long)z * pitch);
    HabcW w{1.f, 0.f, 0.f, 0.f, 0.f};
    if (x < nx) w = habc_weights(z, x, nz, nx, hw, mult != 0, hb[i]);
    out[i] = w.wi;
    out[pl + i] = w.wt;
    out[2 * pl + i] = w.wb;
    out[3 * pl + i] = w.wl;
    out[4 * pl + i] = w.wr;
  }
}
}  // namespace

cudaError_t launch_habc_shares(const sgb_grid& g, const sgb_acoustic_model& m, float* planes, cudaStream_t s) {
  const long long pl = (long long)g.nz * g.pitch;
  long long blocks = (pl + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  habc_shares_kernel<<<(unsigned)blocks, 256, 0, s>>>(g.nz, g.nx, g.pitch, m.habc_width, m.multiple, m.damp, planes);
  return cudaGetLastError();
}

cudaError_t launch_habc_bwd(const sgb_grid& g, const sgb_acoustic_model& m, const sgb_acquisition& q,
                            const Ring& ring, const float* la1, const float* la2, float* lout, const float* uj,
                            const float* ujm1, float* uout, float* grad, const float* ring_in, int t_src,
                            const float* resid, const float* kz, float* grad2, const float* rho_c,
                            float* grad_rho, cudaStream_t s, const float* wpl) {
  HabcBwdArgs a;
  a.wpl = wpl;
  a.kz = kz;
  a.grad2 = grad2;
  a.rho_c = rho_c;
  a.grad_rho = grad_rho;
  a.nz = g.nz;
  a.nx = g.nx;
  a.pitch = g.pitch;
  a.nshots = g.nshots;
  a.hw = m.habc_width;
  a.multiple = m.multiple;
  a.R = m.order / 2;
  a.sstride = (long long)g.nz * g.pitch;
  a.la1 = la1;
  a.la2 = la2;
  a.lout = lout;
  a.uj = uj;
  a.ujm1 = ujm1;
  a.uout = uout;
  a.grad = grad;
  a.k = m.coef + (long long)g.nz * g.pitch;
  a.vp = m.vp;
  a.hb = m.damp;
  a.lamf = 2.f * g.dt / g.h;
  a.muf = (g.dt * g.dt) / (g.h * g.h);
  a.w = fd_weights(m.order);
  a.ring = ring;
  a.ring_in = ring_in;
  a.src_ptr = q.nsrc > 0 ? q.src_ptr : nullptr;
  a.src_z = q.src_z;
  a.src_x = q.src_x;
  a.src_wrow = q.src_wrow;
  a.wavelet = q.wavelet;
  a.nt = q.nt;
  a.t_src = t_src;
  a.rec_row_ptr = q.rec_row_ptr;
  a.rec_x = q.rec_x;
  a.rec_col = q.rec_col;
  a.nch = q.nch;
  a.resid = resid;
  const int R = a.R;
  if (R > HT_H) return cudaErrorInvalidValue;
  const int eq = rho_c != nullptr ? 2 : (kz != nullptr ? 1 : 0);
  if (eq == 2 && R != 1) return cudaErrorInvalidValue;  // variable density: 2nd order only
  // the far tiles (out of reach of every strip: the kernel's own test, per
  // band and per strip) form one block of bands x strips; the rest is the
  // frame around it
  const int HR = R < 2 ? 2 : R;
  a.ntx = (g.nx + HT_X - 1) / HT_X;
  a.nzb = (g.nz + HT_Z - 1) / HT_Z;
  auto near_band = [&](int bz) {
    const int z0 = bz * HT_Z;
    return a.hw > 0 && ((!a.multiple && z0 - HR <= a.hw) || z0 + HT_Z + HR >= a.nz - 1 - a.hw);
  };
  auto near_strip = [&](int sx) {
    const int x0 = sx * HT_X;
    return a.hw > 0 && (x0 - HT_H <= a.hw || x0 + HT_X + HT_H >= a.nx - 1 - a.hw);
  };
  a.fz0 = 0;
  while (a.fz0 < a.nzb && near_band(a.fz0)) ++a.fz0;
  a.fz1 = a.fz0;
  while (a.fz1 < a.nzb && !near_band(a.fz1)) ++a.fz1;
  a.fx0 = 0;
  while (a.fx0 < a.ntx && near_strip(a.fx0)) ++a.fx0;
  a.fx1 = a.fx0;
  while (a.fx1 < a.ntx && !near_strip(a.fx1)) ++a.fx1;
  if (a.fz1 == a.fz0 || a.fx1 == a.fx0) {  // no far tiles
    a.fz0 = a.fz1 = a.nzb;
    a.fx0 = a.fx1 = 0;
  }
  const int nfar = (a.fx1 - a.fx0) * (a.fz1 - a.fz0), nnear = a.ntx * a.nzb - nfar;
  const dim3 gfar((unsigned)(a.fx1 - a.fx0), (unsigned)(a.fz1 - a.fz0), (unsigned)g.nshots);
  const dim3 gnear((unsigned)nnear, 1u, (unsigned)g.nshots);
  // one launch for the tiles out of reach of the strips, one for the rest
  switch (R * 3 + eq) {
#define SGB_TILE2(RR, EQ)                                                                           \
  if constexpr (EQ == 0) {                                                                        \
    if (nfar > 0) habc_bwd_tile_kernel<RR, EQ, false><<<gfar, dim3(32, HT_Z), 0, s>>>(a);         \
    if (nnear > 0) habc_bwd_tile_kernel<RR, EQ, true><<<gnear, dim3(32, HT_Z), 0, s>>>(a);        \
  } else {                                                                                        \
    if (nfar > 0) habc_bwd_tile_kernel_held<RR, EQ, false><<<gfar, dim3(32, HT_Z), 0, s>>>(a);    \
    if (nnear > 0) habc_bwd_tile_kernel_held<RR, EQ, true><<<gnear, dim3(32, HT_Z), 0, s>>>(a);   \
  }
    case 3: SGB_TILE2(1, 0) break;
    case 4: SGB_TILE2(1, 1) break;
    case 5: SGB_TILE2(1, 2) break;
    case 6: SGB_TILE2(2, 0) break;
    case 7: SGB_TILE2(2, 1) break;
    case 9: SGB_TILE2(3, 0) break;
    case 10: SGB_TILE2(3, 1) break;
    case 12: SGB_TILE2(4, 0) break;
    case 13: SGB_TILE2(4, 1) break;
#undef SGB_TILE2
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_habc_step_vjp(const sgb_grid& g, const sgb_acoustic_model& m, const sgb_habc_vjp_io& io,
                                 cudaStream_t s) {
  HabcVjpArgs a;
  a.nz = g.nz;
  a.nx = g.nx;
  a.pitch = g.pitch;
  a.nshots = g.nshots;
  a.hw = m.habc_width;
  a.multiple = m.multiple;
  a.sstride = (long long)g.nz * g.pitch;
  a.u = io.u;
  a.um = io.um;
  a.gy = io.gy;
  a.gu = io.gu;
  a.gum = io.gum;
  a.g = m.coef;
  a.k = m.coef + (long long)g.nz * g.pitch;
  a.kz = io.kz;
  a.rho_c = io.rho_c;
  a.vp = m.vp;
  a.hb = m.damp;
  a.lamf = 2.f * g.dt / g.h;
  a.muf = (g.dt * g.dt) / (g.h * g.h);
  a.w = fd_weights(m.order);
  a.gparam = io.gparam;
  a.gc = io.gvp_oneway;
  a.born_m = io.born_m;
  a.born_u = io.born_u;
  a.born_gu = io.born_gu;
  a.born_gm = io.born_gm;
  a.wi_out = io.wi_out;
  const long long cells = (long long)g.nz * g.nx;
  long long blocks = (cells + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  const int R = m.order / 2;
  const int eq = io.rho_c != nullptr ? 2 : (io.kz != nullptr ? 1 : 0);
  if (eq != 0 && R != 1) return cudaErrorInvalidValue;  // VTI and variable density: 2nd order
  switch (R * 3 + eq) {
    case 3: habc_step_vjp_kernel<1, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 4: habc_step_vjp_kernel<1, 1><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 5: habc_step_vjp_kernel<1, 2><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 6: habc_step_vjp_kernel<2, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 9: habc_step_vjp_kernel<3, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 12: habc_step_vjp_kernel<4, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace sgb
