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
// Two kernels share each reverse step: habc_bwd_interior_kernel takes the
// cells at least hw + R from every strip side (there wi = 1 for the whole
// stencil and no one-way line reaches), with k La1 and U_{j-1} tiles staged
// in shared memory; habc_bwd_kernel takes the remaining frame of cells one
// by one.  The same equations carry the VTI (k Lx + kz Lz, vti_habc2.py),
// variable-density (C D(U), acoustic_rho_habc.py) and Born (the scattered
// field's adjoint against the background's reconstruction,
// acoustic_lsrtm_habc.py) gradients.
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
  // cells [tz0, tz1) x [tx0, tx1) (tx0, tx1 multiples of 4) are done by
  // habc_bwd_interior_kernel; empty (tx1 = tx0) when that kernel is not used
  int tz0, tz1, tx0, tx1;
  // [5][nz][pitch] static shares (wi, wt, wb, wl, wr) of every cell, or null
  const float* __restrict__ wpl;
};

// Is the group of four columns at x0 (a multiple of 4) in row z one of the
// interior kernel's?  The two kernels split the cells with this predicate.
__device__ __forceinline__ bool in_tiled(const HabcBwdArgs& a, int z, int x0) {
  return z >= a.tz0 && z < a.tz1 && x0 >= a.tx0 && x0 + 4 <= a.tx1;
}

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

// Cells of a shot outside the interior kernel's region, numbered rows
// [0, tz0) in full, then rows [tz0, tz1) without columns [tx0, tx1), then
// rows [tz1, nz) in full (all cells when the region is empty).
struct FrameCells {
  int nx, tz0, tz1, tx0, tx1, midw;
  long long top, mid, plane;
  __host__ __device__ FrameCells(const HabcBwdArgs& a)
      : nx(a.nx), tz0(a.tz0), tz1(a.tz1), tx0(a.tx0), tx1(a.tx1), midw(a.tx0 + (a.nx - a.tx1)) {
    top = (long long)tz0 * nx;
    mid = (long long)(tz1 - tz0) * midw;
    plane = top + mid + (long long)(a.nz - tz1) * nx;
  }
  __host__ __device__ void cell(long long r, int& z, int& x) const {
    if (r < top) {
      z = (int)(r / nx);
      x = (int)(r % nx);
    } else if (r < top + mid) {
      const long long q = r - top;
      const int c = (int)(q % midw);
      z = tz0 + (int)(q / midw);
      x = c < tx0 ? c : tx1 + (c - tx0);
    } else {
      const long long q = r - top - mid;
      z = tz1 + (int)(q / nx);
      x = (int)(q % nx);
    }
  }
};

// EQ: 0 plain (acoustic_habc, Born), 1 VTI, 2 variable density -- one
// instantiation per equation, so each carries only its own branches.
template <int R, int EQ>
__global__ void __launch_bounds__(256, 4) habc_bwd_kernel(const HabcBwdArgs a) {
  const FrameCells fc(a);
  const long long plane = fc.plane;
  const long long total = plane * a.nshots;
  const bool mult = a.multiple != 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(i / plane);
    int z, x;
    fc.cell(i - (long long)b * plane, z, x);
    const long long fb = (long long)b * a.sstride;
    const long long o = (long long)z * a.pitch + x;
    const float* l1 = a.la1 + fb;
    const float* l2 = a.la2 + fb;
    const float kq = __ldg(a.k + o);
    // Cells at least hw + R from every strip side: every stencil neighbour
    // lies in the grid with wi = 1 and no one-way line reaches them, so the
    // transpose is the plain 2 La1 + L(k La1) - La2.  With `multiple` the
    // top has no strip, but the stencil must still stay below row 0.
    const int far = a.hw + R;
    const bool interior =
        z >= (mult ? R : far) && a.nz - 1 - z >= far && x >= far && a.nx - 1 - x >= far;
    constexpr bool vti = EQ == 1;
    constexpr bool rho = EQ == 2 && R == 1;
    const float kzq = vti ? __ldg(a.kz + o) : 0.f;
    const float ch = 0.5f * a.w.c[0];  // centre of the 1-D second difference
    const long long pl = (long long)a.nz * a.pitch;
    float v;
    if (rho) {
      // transpose of C D: the cell's own -(bx+ + bx- + bz+ + bz-) C w, plus
      // bx+ C w of the left neighbour, bx- C w of the right one, bz+ C w of
      // the row above and bz- C w of the row below (w = wi La1)
      auto cw = [&](int zz, int xx, int q) -> float {  // C * coefficient q * wi * La1 at (zz, xx)
        if (zz < 0 || zz >= a.nz || xx < 0 || xx >= a.nx) return 0.f;
        const long long oo = (long long)zz * a.pitch + xx;
        const float wi = interior ? 1.f : habc_weights(zz, xx, a.nz, a.nx, a.hw, mult, __ldg(a.hb + oo)).wi;
        return __ldg(a.rho_c + oo) * __ldg(a.rho_c + q * pl + oo) * wi * l1[oo];
      };
      const float wq = interior ? 1.f : habc_weights(z, x, a.nz, a.nx, a.hw, mult, __ldg(a.hb + o)).wi;
      const float sum = __ldg(a.rho_c + pl + o) + __ldg(a.rho_c + 2 * pl + o) + __ldg(a.rho_c + 3 * pl + o) +
                        __ldg(a.rho_c + 4 * pl + o);
      const float own = -sum * __ldg(a.rho_c + o) * wq * l1[o];
      v = 2.f * wq * l1[o] + (own + cw(z, x - 1, 1) + cw(z, x + 1, 2) + cw(z - 1, x, 3) + cw(z + 1, x, 4)) -
          wq * l2[o];
      if (!interior) {
        v += oneway_t<true, true>(a, l1, l2, z, x, z, 1, 0, 0);
        v += oneway_t<true, true>(a, l1, l2, z, x, a.nz - 1 - z, -1, 0, 1);
        v += oneway_t<true, true>(a, l1, l2, z, x, x, 0, 1, 2);
        v += oneway_t<true, true>(a, l1, l2, z, x, a.nx - 1 - x, 0, -1, 3);
      }
    } else if (interior && vti) {
      float lx = ch * kq * l1[o], lz = ch * kzq * l1[o];
      for (int j = 1; j <= R; ++j) {
        const long long up = o - (long long)j * a.pitch, dn = o + (long long)j * a.pitch;
        lx += a.w.c[j] * (__ldg(a.k + o - j) * l1[o - j] + __ldg(a.k + o + j) * l1[o + j]);
        lz += a.w.c[j] * (__ldg(a.kz + up) * l1[up] + __ldg(a.kz + dn) * l1[dn]);
      }
      v = 2.f * l1[o] + lx + lz - l2[o];
    } else if (interior) {
      float lap = a.w.c[0] * kq * l1[o];
      for (int j = 1; j <= R; ++j) {
        const long long up = o - (long long)j * a.pitch, dn = o + (long long)j * a.pitch;
        lap += a.w.c[j] * (__ldg(a.k + up) * l1[up] + __ldg(a.k + dn) * l1[dn] + __ldg(a.k + o - j) * l1[o - j] +
                           __ldg(a.k + o + j) * l1[o + j]);
      }
      v = 2.f * l1[o] + lap - l2[o];
    } else if (vti) {
      // x neighbours weighted by k, z neighbours by kz, each with its interior share
      auto wl = [&](int zz, int xx, const float* kp) -> float {
        if (zz < 0 || zz >= a.nz || xx < 0 || xx >= a.nx) return 0.f;
        const long long oo = (long long)zz * a.pitch + xx;
        const HabcW w = habc_weights(zz, xx, a.nz, a.nx, a.hw, mult, __ldg(a.hb + oo));
        return __ldg(kp + oo) * w.wi * l1[oo];
      };
      const HabcW wq = habc_weights(z, x, a.nz, a.nx, a.hw, mult, __ldg(a.hb + o));
      float lap = ch * (kq + kzq) * wq.wi * l1[o];
      for (int j = 1; j <= R; ++j)
        lap += a.w.c[j] * (wl(z, x - j, a.k) + wl(z, x + j, a.k) + wl(z - j, x, a.kz) + wl(z + j, x, a.kz));
      v = 2.f * wq.wi * l1[o] + lap - wq.wi * l2[o];
      v += oneway_t<true, true>(a, l1, l2, z, x, z, 1, 0, 0);
      v += oneway_t<true, true>(a, l1, l2, z, x, a.nz - 1 - z, -1, 0, 1);
      v += oneway_t<true, true>(a, l1, l2, z, x, x, 0, 1, 2);
      v += oneway_t<true, true>(a, l1, l2, z, x, a.nx - 1 - x, 0, -1, 3);
    } else {
      // interior part: 2 wi La1 + L(k wi La1) - wi La2
      auto kwl = [&](int zz, int xx) -> float {
        if (zz < 0 || zz >= a.nz || xx < 0 || xx >= a.nx) return 0.f;
        const long long oo = (long long)zz * a.pitch + xx;
        const HabcW w = habc_weights(zz, xx, a.nz, a.nx, a.hw, mult, __ldg(a.hb + oo));
        return __ldg(a.k + oo) * w.wi * l1[oo];
      };
      const HabcW wq = habc_weights(z, x, a.nz, a.nx, a.hw, mult, __ldg(a.hb + o));
      float lap = a.w.c[0] * kq * wq.wi * l1[o];
      for (int j = 1; j <= R; ++j)
        lap += a.w.c[j] * (kwl(z - j, x) + kwl(z + j, x) + kwl(z, x - j) + kwl(z, x + j));
      v = 2.f * wq.wi * l1[o] + lap - wq.wi * l2[o];
      // one-way parts of the four sides
      v += oneway_t<true, true>(a, l1, l2, z, x, z, 1, 0, 0);
      v += oneway_t<true, true>(a, l1, l2, z, x, a.nz - 1 - z, -1, 0, 1);
      v += oneway_t<true, true>(a, l1, l2, z, x, x, 0, 1, 2);
      v += oneway_t<true, true>(a, l1, l2, z, x, a.nx - 1 - x, 0, -1, 3);
    }
    // residuals of the records of step j-1 (they sample U_j)
    if (a.resid != nullptr) {
      const int* rp = a.rec_row_ptr + (long long)b * a.nz;
      int lo = rp[z], hi = rp[z + 1];  // receivers of the row, sorted by column
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a.rec_x[mid] < x) lo = mid + 1; else hi = mid;
      }
      for (int q = lo; q < rp[z + 1] && a.rec_x[q] == x; ++q) v += a.resid[(long long)a.rec_col[q] * a.nch];
    }
    a.lout[fb + o] = v;
    // gradient and reconstruction inside the undamped box
    const bool inbox = a.ring.inside(z, x);
    if (inbox) {
      const float* u1 = a.ujm1 + fb;
      float upd;  // k L(U_{j-1}) (VTI: k Lx + kz Lz; variable density: C D(U))
      if (rho) {
        const float u0 = u1[o];
        const float dxp = ldz(u1, z, x + 1, a.nz, a.nx, a.pitch) - u0, dxn = u0 - ldz(u1, z, x - 1, a.nz, a.nx, a.pitch);
        const float dzp = ldz(u1, z + 1, x, a.nz, a.nx, a.pitch) - u0, dzn = u0 - ldz(u1, z - 1, x, a.nz, a.nx, a.pitch);
        const float bxp = __ldg(a.rho_c + pl + o), bxn = __ldg(a.rho_c + 2 * pl + o);
        const float bzp = __ldg(a.rho_c + 3 * pl + o), bzn = __ldg(a.rho_c + 4 * pl + o);
        const float D = bxp * dxp - bxn * dxn + bzp * dzp - bzn * dzn;
        const float C = __ldg(a.rho_c + o);
        const long long fs = (long long)a.nshots * a.sstride;  // one gradient field
        float* gr = a.grad_rho + fb + o;
        gr[0] += v * D;
        gr[fs] += v * C * dxp;
        gr[2 * fs] -= v * C * dxn;
        gr[3 * fs] += v * C * dzp;
        gr[4 * fs] -= v * C * dzn;
        upd = C * D;
      } else if (vti) {
        float Lx = ch * u1[o], Lz = ch * u1[o];
        for (int j = 1; j <= R; ++j) {
          Lx += a.w.c[j] * (ldz(u1, z, x - j, a.nz, a.nx, a.pitch) + ldz(u1, z, x + j, a.nz, a.nx, a.pitch));
          Lz += a.w.c[j] * (ldz(u1, z - j, x, a.nz, a.nx, a.pitch) + ldz(u1, z + j, x, a.nz, a.nx, a.pitch));
        }
        a.grad[fb + o] += v * Lx;  // dJ/dk
        a.grad2[fb + o] += v * Lz;  // dJ/dkz
        upd = kq * Lx + kzq * Lz;
      } else {
        float L = a.w.c[0] * u1[o];
        for (int j = 1; j <= R; ++j)
          L += a.w.c[j] * (ldz(u1, z - j, x, a.nz, a.nx, a.pitch) + ldz(u1, z + j, x, a.nz, a.nx, a.pitch) +
                           ldz(u1, z, x - j, a.nz, a.nx, a.pitch) + ldz(u1, z, x + j, a.nz, a.nx, a.pitch));
        a.grad[fb + o] += v * kq * L;  // times 2 / vp in the shot reduction (dJ/dvp)
        upd = kq * L;
      }
      if (a.uout != nullptr) {
        float ujv = a.uj[fb + o];
        if (a.src_ptr != nullptr) {
          for (int q = a.src_ptr[b]; q < a.src_ptr[b + 1]; ++q)
            if (a.src_z[q] == z && a.src_x[q] == x) ujv -= a.wavelet[(long long)a.src_wrow[q] * a.nt + a.t_src];
        }
        a.uout[fb + o] = 2.f * u1[o] - ujv + upd;
      }
    } else {
      if (rho) {
        // the box's one-cell rim: the half-point buoyancy terms that reach
        // into the box (their U values are the box's and the saved ring's),
        // so that dJ/drho is complete at the box's edge cells
        const bool xr = a.ring.inside(z, x + 1), xl = a.ring.inside(z, x - 1);
        const bool zd = a.ring.inside(z + 1, x), zu = a.ring.inside(z - 1, x);
        if (xr || xl || zd || zu) {
          const float* u1 = a.ujm1 + fb;
          const float u0 = u1[o], vC = v * __ldg(a.rho_c + o);
          const long long fs = (long long)a.nshots * a.sstride;
          float* gr = a.grad_rho + fb + o;
          if (xr) gr[fs] += vC * (u1[o + 1] - u0);
          if (xl) gr[2 * fs] -= vC * (u0 - u1[o - 1]);
          if (zd) gr[3 * fs] += vC * (u1[o + a.pitch] - u0);
          if (zu) gr[4 * fs] -= vC * (u0 - u1[o - a.pitch]);
        }
      }
      if (a.uout != nullptr) {  // the saved ring around the box, 0 beyond it
        const int ri = a.ring.index(z, x);
        a.uout[fb + o] = (ri >= 0 && a.ring_in != nullptr) ? a.ring_in[(long long)b * a.ring.size + ri] : 0.f;
      }
    }
  }
}

// Interior cells (at least hw + R from every strip side, inside the box;
// plain or VTI equation, not variable density): the transpose
// 2 La1 + L(k La1) - La2, the gradient term and the reconstruction, with
// k La1 and U_{j-1} of an 8 x 128 tile plus its halo staged once in shared
// memory.  Block (32, 8): warp w owns row z0 + w, lane l columns x0 + 4l.
constexpr int HT_Z = 8, HT_X = 128, HT_H = 4;  // rows, columns, column halo (>= R)
template <int R, bool VTI>
__global__ void __launch_bounds__(256) habc_bwd_interior_kernel(const HabcBwdArgs a) {
  constexpr int ROWS = HT_Z + 2 * R, W = HT_X + 2 * HT_H;
  __shared__ __align__(16) float s_kl[ROWS][W];              // k La1 (VTI: kx La1)
  __shared__ __align__(16) float s_kzl[VTI ? ROWS : 1][W];   // VTI: kz La1
  __shared__ __align__(16) float s_u[ROWS][W];
  const int b = blockIdx.z;
  const int z0 = a.tz0 + blockIdx.y * HT_Z, x0 = a.tx0 + blockIdx.x * HT_X;
  const long long fb = (long long)b * a.sstride;
  const float* l1 = a.la1 + fb;
  const float* u1 = a.ujm1 + fb;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  // stage: rows z0-R .. z0+HT_Z+R-1, columns x0-4 .. x0+131 (zeros off the grid)
  for (int c = tid; c < ROWS * (W / 4); c += 256) {
    const int rr = c / (W / 4), cc = c - rr * (W / 4);
    const int z = z0 - R + rr, x = x0 - HT_H + 4 * cc;
    float4 kl = make_float4(0.f, 0.f, 0.f, 0.f), uu = kl, kzl = kl;
    if (z >= 0 && z < a.nz && x >= 0 && x + 4 <= a.pitch) {
      const long long o = (long long)z * a.pitch + x;
      const float4 k4 = __ldg(reinterpret_cast<const float4*>(a.k + o));
      const float4 l4 = *reinterpret_cast<const float4*>(l1 + o);
      kl = make_float4(k4.x * l4.x, k4.y * l4.y, k4.z * l4.z, k4.w * l4.w);
      if (VTI) {
        const float4 q4 = __ldg(reinterpret_cast<const float4*>(a.kz + o));
        kzl = make_float4(q4.x * l4.x, q4.y * l4.y, q4.z * l4.z, q4.w * l4.w);
      }
      uu = *reinterpret_cast<const float4*>(u1 + o);
    }
    *reinterpret_cast<float4*>(&s_kl[rr][4 * cc]) = kl;
    if (VTI) *reinterpret_cast<float4*>(&s_kzl[rr][4 * cc]) = kzl;
    *reinterpret_cast<float4*>(&s_u[rr][4 * cc]) = uu;
  }
  __syncthreads();
  const int z = z0 + threadIdx.y, x = x0 + 4 * threadIdx.x;
  if (!in_tiled(a, z, x)) return;
  const int rr = R + threadIdx.y, cx = HT_H + 4 * threadIdx.x;
  const long long o = (long long)z * a.pitch + x;
  const float4 l2 = *reinterpret_cast<const float4*>(a.la2 + fb + o);
  const float4 l1c = *reinterpret_cast<const float4*>(l1 + o);
  const float4 k4 = __ldg(reinterpret_cast<const float4*>(a.k + o));
  float v[4], L[4], Lz[4];  // VTI: L = Lx(U), Lz = Lz(U)
  const float ch = 0.5f * a.w.c[0];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    if (VTI) {  // the per-cell VTI interior path, term by term
      float lx = ch * s_kl[rr][cx + m], lz = ch * s_kzl[rr][cx + m];
      float ux = ch * s_u[rr][cx + m], uz = ch * s_u[rr][cx + m];
#pragma unroll
      for (int j = 1; j <= R; ++j) {
        lx += a.w.c[j] * (s_kl[rr][cx + m - j] + s_kl[rr][cx + m + j]);
        lz += a.w.c[j] * (s_kzl[rr - j][cx + m] + s_kzl[rr + j][cx + m]);
        ux += a.w.c[j] * (s_u[rr][cx + m - j] + s_u[rr][cx + m + j]);
        uz += a.w.c[j] * (s_u[rr - j][cx + m] + s_u[rr + j][cx + m]);
      }
      v[m] = 2.f * comp(l1c, m) + lx + lz - comp(l2, m);
      L[m] = ux;
      Lz[m] = uz;
    } else {
      float lap = a.w.c[0] * s_kl[rr][cx + m];
      float lu = a.w.c[0] * s_u[rr][cx + m];
#pragma unroll
      for (int j = 1; j <= R; ++j) {
        lap += a.w.c[j] * (s_kl[rr - j][cx + m] + s_kl[rr + j][cx + m] + s_kl[rr][cx + m - j] + s_kl[rr][cx + m + j]);
        lu += a.w.c[j] * (s_u[rr - j][cx + m] + s_u[rr + j][cx + m] + s_u[rr][cx + m - j] + s_u[rr][cx + m + j]);
      }
      v[m] = 2.f * comp(l1c, m) + lap - comp(l2, m);
      L[m] = lu;
      Lz[m] = 0.f;
    }
  }
  // residuals of the records of step j-1 in this row
  if (a.resid != nullptr) {
    const int* rp = a.rec_row_ptr + (long long)b * a.nz;
    int lo = rp[z], hi = rp[z + 1];  // receivers of the row, sorted by column
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
  float4* gp = reinterpret_cast<float4*>(a.grad + fb + o);
  const float4 g0 = *gp;
  float4 kz4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (VTI) {  // dJ/dkx += La Lx(U), dJ/dkz += La Lz(U)
    *gp = make_float4(g0.x + v[0] * L[0], g0.y + v[1] * L[1], g0.z + v[2] * L[2], g0.w + v[3] * L[3]);
    float4* gq = reinterpret_cast<float4*>(a.grad2 + fb + o);
    const float4 h0 = *gq;
    *gq = make_float4(h0.x + v[0] * Lz[0], h0.y + v[1] * Lz[1], h0.z + v[2] * Lz[2], h0.w + v[3] * Lz[3]);
    kz4 = __ldg(reinterpret_cast<const float4*>(a.kz + o));
  } else {
    *gp = make_float4(g0.x + v[0] * k4.x * L[0], g0.y + v[1] * k4.y * L[1], g0.z + v[2] * k4.z * L[2],
                      g0.w + v[3] * k4.w * L[3]);
  }
  if (a.uout != nullptr) {
    const float4 uj = *reinterpret_cast<const float4*>(a.uj + fb + o);
    float ujv[4] = {uj.x, uj.y, uj.z, uj.w};
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
    float uo[4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
      uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + (VTI ? comp(k4, m) * L[m] + comp(kz4, m) * Lz[m] : comp(k4, m) * L[m]);
    *reinterpret_cast<float4*>(a.uout + fb + o) = make_float4(uo[0], uo[1], uo[2], uo[3]);
  }
}


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
// The plain / VTI / Born reverse step in one launch, tile 8 x 128 with block
// (32, 8) (lane: four columns).  La_j = 2 wi La1 + L(k wi La1) - wi La2 (VTI:
// x neighbours by kx, z neighbours by kz) from shared-memory tiles of
// k wi La1 and U_{j-1}; tiles within reach of a strip also stage La1 and La2
// (two-row halo) and add the one-way transposes of the four sides, with each
// cell's interior and side shares read from the five planes that
// habc_shares_kernel fills once per reverse loop; then the receiver
// residuals, the gradient term and the reconstruction inside the box, the
// saved ring (or 0) outside it.
template <int R, bool VTI, bool NEAR>
__global__ void __launch_bounds__(256) habc_bwd_tile_kernel(const HabcBwdArgs a) {
  // row halo: the stencil's R, and 2 for the one-way lines (q - d, q - 2d)
  constexpr int HR = R < 2 ? 2 : R;
  constexpr int ROWS = HT_Z + 2 * HR, W = HT_X + 2 * HT_H;
  __shared__ __align__(16) float s_kl[ROWS][W];             // k wi La1 (VTI: kx wi La1)
  __shared__ __align__(16) float s_kzl[VTI ? ROWS : 1][W];  // VTI: kz wi La1
  __shared__ __align__(16) float s_u[ROWS][W];
  __shared__ __align__(16) float s_l1[NEAR ? ROWS : 1][W];  // La1 and La2 (tiles near a strip only)
  __shared__ __align__(16) float s_l2[NEAR ? ROWS : 1][W];
  const int b = blockIdx.z;
  const int z0 = blockIdx.y * HT_Z, x0 = blockIdx.x * HT_X;
  const long long fb = (long long)b * a.sstride;
  const float* l1 = a.la1 + fb;
  const float* u1 = a.ujm1 + fb;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int hw = a.hw;
  const bool mult = a.multiple != 0;
  const long long pl = (long long)a.nz * a.pitch;
  // does any cell of the tile or its halo have an interior share below 1, or
  // lie within reach of a one-way line (depth <= hw)?
  const bool near = hw > 0 && ((!mult && z0 - HR <= hw) || z0 + HT_Z + HR >= a.nz - 1 - hw ||
                                x0 - HT_H <= hw || x0 + HT_X + HT_H >= a.nx - 1 - hw);
  // two launches share the grid: the NEAR instantiation takes the tiles
  // within reach of a strip, the other the rest (with none of the strip code)
  if (near != NEAR) return;
  auto wi_at = [&](int z, int x) -> float {
    if (!near) return 1.f;
    const long long oo = (long long)z * a.pitch + x;
    if (a.wpl != nullptr) return __ldg(a.wpl + oo);
    const float bb = __ldg(a.hb + oo);  // b = 0: no side share, wi = 1
    return bb == 0.f ? 1.f : habc_weights(z, x, a.nz, a.nx, hw, mult, bb).wi;
  };
  for (int c = tid; c < ROWS * (W / 4); c += 256) {
    const int rr = c / (W / 4), cc = c - rr * (W / 4);
    const int z = z0 - HR + rr, x = x0 - HT_H + 4 * cc;
    float kl[4] = {0.f, 0.f, 0.f, 0.f}, kzl[4] = {0.f, 0.f, 0.f, 0.f}, uu[4] = {0.f, 0.f, 0.f, 0.f};
    float r1[4] = {0.f, 0.f, 0.f, 0.f}, r2[4] = {0.f, 0.f, 0.f, 0.f};
    if (z >= 0 && z < a.nz && x >= 0 && x < a.nx) {
      const long long o = (long long)z * a.pitch + x;
      const float4 k4 = __ldg(reinterpret_cast<const float4*>(a.k + o));
      const float4 l4 = *reinterpret_cast<const float4*>(l1 + o);
      const float4 q4 = VTI ? __ldg(reinterpret_cast<const float4*>(a.kz + o)) : k4;
      const float4 v4 = *reinterpret_cast<const float4*>(u1 + o);
      const float4 m4 = NEAR ? *reinterpret_cast<const float4*>(a.la2 + fb + o) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        if (x + m < a.nx) {
          const float w = wi_at(z, x + m);
          kl[m] = comp(k4, m) * w * comp(l4, m);
          if (VTI) kzl[m] = comp(q4, m) * w * comp(l4, m);
          uu[m] = comp(v4, m);
          r1[m] = comp(l4, m);
          r2[m] = comp(m4, m);
        }
      }
    }
    *reinterpret_cast<float4*>(&s_kl[rr][4 * cc]) = make_float4(kl[0], kl[1], kl[2], kl[3]);
    if (VTI) *reinterpret_cast<float4*>(&s_kzl[rr][4 * cc]) = make_float4(kzl[0], kzl[1], kzl[2], kzl[3]);
    *reinterpret_cast<float4*>(&s_u[rr][4 * cc]) = make_float4(uu[0], uu[1], uu[2], uu[3]);
    if constexpr (NEAR) {
      *reinterpret_cast<float4*>(&s_l1[rr][4 * cc]) = make_float4(r1[0], r1[1], r1[2], r1[3]);
      *reinterpret_cast<float4*>(&s_l2[rr][4 * cc]) = make_float4(r2[0], r2[1], r2[2], r2[3]);
    }
  }
  __syncthreads();
  const int z = z0 + threadIdx.y, x = x0 + 4 * threadIdx.x;
  if (z >= a.nz || x >= a.nx) return;
  const int rr = HR + threadIdx.y, cx = HT_H + 4 * threadIdx.x;
  const long long o = (long long)z * a.pitch + x;
  const float4 l2v = *reinterpret_cast<const float4*>(a.la2 + fb + o);
  const float4 l1c = *reinterpret_cast<const float4*>(l1 + o);
  const float4 k4 = __ldg(reinterpret_cast<const float4*>(a.k + o));
  const float4 kz4 = VTI ? __ldg(reinterpret_cast<const float4*>(a.kz + o)) : k4;
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
  // the one-way sums of the four cells: one copy of the code for every
  // (cell, side) pair (not unrolled, so the kernel stays small)
  float4 ow4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (NEAR) {
#pragma unroll 1
    for (int t = 0; t < 16; ++t) {
      const int m = t >> 2, sd = t & 3;
      const int xm = x + m;
      if (xm >= a.nx) continue;
      const int dq = sd == 0 ? z : sd == 1 ? a.nz - 1 - z : sd == 2 ? xm : a.nx - 1 - xm;
      if (dq > hw) continue;
      const int sz = sd == 0 ? 1 : sd == 1 ? -1 : 0, sx = sd == 2 ? 1 : sd == 3 ? -1 : 0;
      set_comp(ow4, m, comp(ow4, m) + oneway(sd, dq, sz, sx, xm, cx + m));
    }
  }
  const float ch = 0.5f * a.w.c[0];
  float v[4], L[4], Lz[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int xm = x + m;
    const float wq = (xm < a.nx) ? wi_at(z, xm) : 0.f;
    const float ow = NEAR ? comp(ow4, m) : 0.f;
    float lap, lu, luz = 0.f;
    if (VTI) {
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
  const bool row_in = z >= a.ring.iz0 && z < a.ring.iz1;
  float uo[4] = {0.f, 0.f, 0.f, 0.f};
  float ujv[4] = {0.f, 0.f, 0.f, 0.f};
  if (a.uout != nullptr && row_in) {
    const float4 uj = *reinterpret_cast<const float4*>(a.uj + fb + o);
    ujv[0] = uj.x; ujv[1] = uj.y; ujv[2] = uj.z; ujv[3] = uj.w;
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
  if (row_in && x >= a.ring.ix0 && x + 3 < a.ring.ix1) {
    // all four columns inside the box: vector gradient update and reconstruction
    float4* gp = reinterpret_cast<float4*>(a.grad + fb + o);
    const float4 g0 = *gp;
    if (VTI) {
      *gp = make_float4(g0.x + v[0] * L[0], g0.y + v[1] * L[1], g0.z + v[2] * L[2], g0.w + v[3] * L[3]);
      float4* gq = reinterpret_cast<float4*>(a.grad2 + fb + o);
      const float4 h0 = *gq;
      *gq = make_float4(h0.x + v[0] * Lz[0], h0.y + v[1] * Lz[1], h0.z + v[2] * Lz[2], h0.w + v[3] * Lz[3]);
    } else {
      *gp = make_float4(g0.x + v[0] * k4.x * L[0], g0.y + v[1] * k4.y * L[1], g0.z + v[2] * k4.z * L[2],
                        g0.w + v[3] * k4.w * L[3]);
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
      if (VTI) {
        a.grad[fb + om] += v[m] * L[m];
        a.grad2[fb + om] += v[m] * Lz[m];
        uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + kk * L[m] + comp(kz4, m) * Lz[m];
      } else {
        a.grad[fb + om] += v[m] * kk * L[m];
        uo[m] = 2.f * s_u[rr][cx + m] - ujv[m] + kk * L[m];
      }
    } else if (a.uout != nullptr) {
      const int ri = a.ring.index(z, xm);
      uo[m] = (ri >= 0 && a.ring_in != nullptr) ? a.ring_in[(long long)b * a.ring.size + ri] : 0.f;
    }
  }
  if (a.uout != nullptr) *reinterpret_cast<float4*>(a.uout + fb + o) = make_float4(uo[0], uo[1], uo[2], uo[3]);
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
  const int R = a.R, far = a.hw + R;
  const bool vti = kz != nullptr;
  if (rho_c == nullptr && R <= HT_H) {
    // plain / VTI / Born: every cell in tiles
    a.tz0 = a.tz1 = a.tx0 = a.tx1 = 0;
    const dim3 grid((unsigned)((g.nx + HT_X - 1) / HT_X), (unsigned)((g.nz + HT_Z - 1) / HT_Z), (unsigned)g.nshots);
    switch (R * 2 + (vti ? 1 : 0)) {
#define SGB_TILE2(RR, V)                                                    \
  habc_bwd_tile_kernel<RR, V, false><<<grid, dim3(32, HT_Z), 0, s>>>(a); \
  if (a.hw > 0) habc_bwd_tile_kernel<RR, V, true><<<grid, dim3(32, HT_Z), 0, s>>>(a);
      case 2: SGB_TILE2(1, false) break;
      case 3: SGB_TILE2(1, true) break;
      case 4: SGB_TILE2(2, false) break;
      case 5: SGB_TILE2(2, true) break;
      case 6: SGB_TILE2(3, false) break;
      case 7: SGB_TILE2(3, true) break;
      case 8: SGB_TILE2(4, false) break;
      case 9: SGB_TILE2(4, true) break;
#undef SGB_TILE2
      default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
  // variable density: the tiled interior kernel does not apply (rho_c set),
  // so the per-cell kernel takes every cell
  a.tz0 = a.multiple ? R : far;
  a.tz1 = g.nz - far;
  a.tx0 = (far + 3) / 4 * 4;
  a.tx1 = (g.nx - far) / 4 * 4;
  const bool tiled = rho_c == nullptr && R <= HT_H && a.tz1 > a.tz0 && a.tx1 > a.tx0 && a.tz0 >= R &&
                     a.tz1 + R <= g.nz;
  if (!tiled) a.tz0 = a.tz1 = a.tx0 = a.tx1 = 0;
  if (tiled) {
    // the box must cover the region (the gradient and the reconstruction
    // are written there unconditionally)
    if (a.tz0 < ring.iz0 || a.tz1 > ring.iz1 || a.tx0 < ring.ix0 || a.tx1 > ring.ix1) {
      a.tz0 = a.tz1 = a.tx0 = a.tx1 = 0;
    } else {
      const dim3 grid((unsigned)((a.tx1 - a.tx0 + HT_X - 1) / HT_X), (unsigned)((a.tz1 - a.tz0 + HT_Z - 1) / HT_Z),
                      (unsigned)g.nshots);
      switch (R * 2 + (vti ? 1 : 0)) {
        case 2: habc_bwd_interior_kernel<1, false><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 3: habc_bwd_interior_kernel<1, true><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 4: habc_bwd_interior_kernel<2, false><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 5: habc_bwd_interior_kernel<2, true><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 6: habc_bwd_interior_kernel<3, false><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 7: habc_bwd_interior_kernel<3, true><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 8: habc_bwd_interior_kernel<4, false><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
        case 9: habc_bwd_interior_kernel<4, true><<<grid, dim3(32, HT_Z), 0, s>>>(a); break;
      }
    }
  }
  const long long total = FrameCells(a).plane * g.nshots;
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  const int eq = rho_c != nullptr ? 2 : (kz != nullptr ? 1 : 0);
  if (eq == 2 && a.R != 1) return cudaErrorInvalidValue;  // variable density: 2nd order only
  switch (a.R * 3 + eq) {
    case 3: habc_bwd_kernel<1, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 4: habc_bwd_kernel<1, 1><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 5: habc_bwd_kernel<1, 2><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 6: habc_bwd_kernel<2, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 7: habc_bwd_kernel<2, 1><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 9: habc_bwd_kernel<3, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 10: habc_bwd_kernel<3, 1><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 12: habc_bwd_kernel<4, 0><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case 13: habc_bwd_kernel<4, 1><<<(unsigned)blocks, 256, 0, s>>>(a); break;
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
