// The hybrid absorbing boundary's blend of one cell (acoustic_habc.py:79-204),
// shared by the HABC step kernels: the one-way extrapolation of each side
// along its inward normal, blended with the interior value y by the weight
// b, under the reference's mask precedence and corner diagonals.  A Tile
// gives U(z, x) (the current field) and P(z, x) (the previous field); Args
// carries nz, nx, pitch, hw, multiple, vp, hb (the weight b), lamf, muf.
#pragma once

#include "sgb_common.cuh"

namespace sgb {

// One side of the hybrid ABC at (z, x): one-way extrapolation along the
// inward step (dz, dx) blended with the interior value y
// (acoustic_habc.py:79-101).  At depth hw-1 the second inward neighbour
// wraps to the edge cell (ze, xe), as torch.roll does on the 51-deep slab.
template <class Tile>
__device__ __forceinline__ float habc_side(const Tile& T, int z, int x, int dz, int dx, int depth,
                                           int hw, int ze, int xe, float y, float c, float b,
                                           float lamf, float muf) {
  const float lam = c * lamf;
  const float mu = c * c * muf;
  const float U0 = T.U(z, x);
  const float U1 = T.U(z + dz, x + dx);
  const float U2 = (depth + 2 <= hw) ? T.U(z + 2 * dz, x + 2 * dx) : T.U(ze, xe);
  const float P0 = T.P(z, x);
  const float P1 = T.P(z + dz, x + dx);
  const float t1 = (2.f - lam - mu) * U0;
  const float t2 = (lam + 2.f * mu) * U1;
  const float t3 = -mu * U2;
  const float t4 = (lam - 1.f) * P0;
  const float t5 = -lam * P1;
  const float uo = t1 + t2 + t3 + t4 + t5;
  return uo * b + (1.f - b) * y;
}

// Mask precedence and corner diagonals of acoustic_habc.py:167-202.
template <class Tile, class Args>
__device__ __forceinline__ float habc_point(const Tile& T, const Args& a, int z, int x, float y) {
  const int hw = a.hw, nz = a.nz, nx = a.nx;
  const int dT = z, dB = nz - 1 - z, dL = x, dR = nx - 1 - x;
  if (!(dT < hw || dB < hw || dL < hw || dR < hw)) return y;
  const bool mult = a.multiple != 0;
  const bool top = !mult && dT < hw && dT <= dL && dT <= dR;
  const bool bot = dB < hw && dB <= dL && dB <= dR;
  const bool lft = dL < hw && ((mult && z < hw) || ((z >= hw || dL <= z) && (dB >= hw || dL <= dB)));
  const bool rgt = dR < hw && ((mult && z < hw) || ((z >= hw || dR <= z) && (dB >= hw || dR <= dB)));
  const bool tl = !mult && z < hw && x == z;
  const bool tr = !mult && z < hw && x == nx - hw + z;
  const bool bl = z >= nz - hw && x == z - (nz - hw);
  const bool br = z >= nz - hw && x == nx - hw + z - (nz - hw);
  const long long p = (long long)z * a.pitch + x;
  const float c = a.vp[p], b = a.hb[p];
  float yT = 0.f, yB = 0.f, yL = 0.f, yR = 0.f;
  if (top || tl || tr) yT = habc_side(T, z, x, 1, 0, dT, hw, 0, x, y, c, b, a.lamf, a.muf);
  if (bot || bl || br) yB = habc_side(T, z, x, -1, 0, dB, hw, nz - 1, x, y, c, b, a.lamf, a.muf);
  if (lft || tl || bl) yL = habc_side(T, z, x, 0, 1, dL, hw, z, 0, y, c, b, a.lamf, a.muf);
  if (rgt || tr || br) yR = habc_side(T, z, x, 0, -1, dR, hw, z, nx - 1, y, c, b, a.lamf, a.muf);
  float v = y;
  if (top) v = yT;
  if (bot) v = yB;
  if (lft) v = yL;
  if (rgt) v = yR;
  if (tl) v = 0.5f * yT + 0.5f * yL;
  if (tr) v = 0.5f * yT + 0.5f * yR;
  if (bl) v = 0.5f * yB + 0.5f * yL;
  if (br) v = 0.5f * yB + 0.5f * yR;
  return v;
}

}  // namespace sgb
