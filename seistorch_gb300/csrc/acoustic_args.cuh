// Kernel argument blocks of the acoustic kernels (filled by capi.cu).
#pragma once

#include <cuda.h>

#include "sgb_common.cuh"

namespace sgb {

// Forward step: un = step(u, um) + sources; records / ring / illumination.
struct AcStepArgs {
  int nz, nx, pitch, nshots, ntx;
  long long sstride;
  const float* __restrict__ u;
  const float* __restrict__ um;
  float* __restrict__ un;
  const float* __restrict__ g;
  const float* __restrict__ k;
  FdWeights w;
  // HABC (acoustic_habc.py:79-204)
  const float* __restrict__ vp;
  const float* __restrict__ hb;
  float lamf, muf;  // 2 dt / h, dt^2 / h^2
  int hw, multiple;
  // sources of this step (rnn.py:196-199, source.py:47-57)
  const int* __restrict__ src_ptr;
  const int* __restrict__ src_z;
  const int* __restrict__ src_x;
  const int* __restrict__ src_wrow;
  const float* __restrict__ wavelet;
  int nt, t;
  // receivers of this step (probe.py:42-44)
  const int* __restrict__ rec_row_ptr;
  const int* __restrict__ rec_x;
  const int* __restrict__ rec_col;
  int nrec, nch;
  float* __restrict__ records;  // records + t*nrec*nch (channel 0)
  float* __restrict__ illum;
  Ring ring;
  // Born modelling (acoustic_lsrtm_habc.py:11-30): the background step
  // writes born_out = born_m k L(u) (per shot); the scattered step adds
  // born_in to its interior update before the boundary blend.  Null otherwise.
  const float* __restrict__ born_m;  // [nz][pitch]
  float* __restrict__ born_out;      // [nshots][nz][pitch]
  const float* __restrict__ born_in;  // [nshots][nz][pitch]
  // VTI (vti_habc2.py:26-56): with kz set, the update is
  // 2u - u- + k Lx(u) + kz Lz(u) (k, kz: the x and z coefficient planes)
  const float* __restrict__ kz;
  // variable density (acoustic_rho_habc.py:34-58): with rho_c set (five
  // planes C, bx+, bx-, bz+, bz-), the update is 2u - u- + C (bx+ (u[x+1] -
  // u) - bx- (u - u[x-1]) + bz+ (u[z+1] - u) - bz- (u - u[z-1])); order 2
  const float* __restrict__ rho_c;
  int* status;
};

// Single-step vector-Jacobian product (PML).
struct AcVjpArgs {
  int nz, nx, pitch, nshots, ntx;
  long long sstride;
  const float* __restrict__ u;    // h1 (stencil)
  const float* __restrict__ gy;   // dJ/dy (stencil through k)
  const float* __restrict__ gh1;  // dJ/d(h1 passthrough) or null
  float* __restrict__ gu;
  float* __restrict__ gum;
  float* __restrict__ gvp;        // [nz][pitch] += sum_b gy L(u) 2k/vp
  const float* __restrict__ g;
  const float* __restrict__ k;
  const float* __restrict__ vp;
  FdWeights w;
};

// Streaming forward step (PML): TMA-fed per-warp strips.
struct AcStreamArgs {
  int nz, nx, pitch, nshots, ntx, zc, nzc;
  int nseg, tpu;  // tiles per column band and per unit (1: every tile stands alone)
  const float* __restrict__ um;   // U_{n-1}
  const float* __restrict__ g;    // coefficient planes
  const float* __restrict__ k;
  const int* __restrict__ src_zr;
  const int* __restrict__ rec_zr;
  long long sstride;
  float* __restrict__ un;
  FdWeights w;
  const int* __restrict__ src_ptr;
  const int* __restrict__ src_z;
  const int* __restrict__ src_x;
  const int* __restrict__ src_wrow;
  const float* __restrict__ wavelet;
  int nt, t;
  const int* __restrict__ rec_row_ptr;
  const int* __restrict__ rec_x;
  const int* __restrict__ rec_col;
  int nrec, nch;
  float* __restrict__ records;
  float* __restrict__ illum;
  Ring ring;
  // boundary ring of the input field U_n (read-only in this launch) into
  // ring_dst [nshots][ring.size], or null; single-grid launches only
  const float* __restrict__ ring_src;
  float* __restrict__ ring_dst;
  int* status;
  // HABC family (single-grid launches of the HABC instantiation only): the
  // input field for strip neighbours outside the staged box, the blend
  // (acoustic_habc.py:79-204), and the equation variants of AcStepArgs
  const float* __restrict__ u;
  const float* __restrict__ vp;
  const float* __restrict__ hb;
  float lamf, muf;
  int hw, multiple;
  const float* __restrict__ kz;
  const float* __restrict__ rho_c;
  const float* __restrict__ born_m;
  float* __restrict__ born_out;
  const float* __restrict__ born_in;
};

// Forward steps of up to MAXG grids in one launch (tiles numbered group
// after group from tile0[g]); MAXG = 1 is the single-grid path.
constexpr int MAX_BATCH_GROUPS = 8;
template <int MAXG>
struct AcFwdBatch {
  CUtensorMap tm_u[MAXG];
  CUtensorMap tm_um[MAXG];
  AcStreamArgs g[MAXG];
  int tile0[MAXG + 1];
  int ngroups;
};

// Fused adjoint step (PML) of the TMA tile pipeline; the adjoint is carried
// as nu = k * Lambda.
struct AcBwdStreamArgs {
  int nz, nx, pitch, nshots, ntx, zc, nzc;
  int nseg, tpu;
  const float* __restrict__ unext;  // U_j
  const float* __restrict__ n2;     // nu_{j+2}
  const float* __restrict__ g;
  const float* __restrict__ k;
  const int* __restrict__ src_zr;
  const int* __restrict__ rec_zr;
  long long sstride;
  float* __restrict__ lout;       // nu_j
  float* __restrict__ uout;       // U_{j-2}
  float* __restrict__ grad_shot;  // read through TMA, written here
  FdWeights w;
  int do_recon;
  Ring ring;  // U_{j-2} is reconstructed inside the box; its ring cells come from ring_in
  const float* __restrict__ ring_in;  // ring of U_{j-2} [nshots][ring.size], or null
  const int* __restrict__ src_ptr;
  const int* __restrict__ src_z;
  const int* __restrict__ src_x;
  const int* __restrict__ src_wrow;
  const float* __restrict__ wavelet;
  int nt, t_src;
  const int* __restrict__ rec_row_ptr;
  const int* __restrict__ rec_x;
  const int* __restrict__ rec_col;
  int nrec, nch;
  const float* __restrict__ resid;
  int* status;
};

}  // namespace sgb
