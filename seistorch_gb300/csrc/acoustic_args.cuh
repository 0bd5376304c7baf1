// Kernel argument blocks of the acoustic kernels (filled by capi.cu).
#pragma once

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
  float* __restrict__ ring_out;  // [nshots][ring.size] of U_{n+1}, or null
  Ring ring;
  int* status;
};

// Fused adjoint step (PML): Lambda_j, U_{j-2} and the gradient term.
struct AcBwdArgs {
  int nz, nx, pitch, nshots, ntx;
  long long sstride;
  const float* __restrict__ ucur;   // U_{j-1} (stencil)
  const float* __restrict__ unext;  // U_j
  float* __restrict__ uout;         // U_{j-2}
  const float* __restrict__ l1;     // Lambda_{j+1} (stencil)
  const float* __restrict__ l2;     // Lambda_{j+2}
  float* __restrict__ lout;         // Lambda_j
  const float* __restrict__ g;
  const float* __restrict__ k;
  FdWeights w;
  float* __restrict__ grad_shot;  // [nshots][nz][pitch]
  // reconstruction
  int do_recon;
  const float* __restrict__ ring_in;  // [nshots][ring.size] of U_{j-2}, or null (U_{j-2} = 0)
  Ring ring;
  // forward sources at time j-1 (subtracted from U_j)
  const int* __restrict__ src_ptr;
  const int* __restrict__ src_z;
  const int* __restrict__ src_x;
  const int* __restrict__ src_wrow;
  const float* __restrict__ wavelet;
  int nt, t_src;
  // adjoint sources: dJ/d records at time j-1
  const int* __restrict__ rec_row_ptr;
  const int* __restrict__ rec_x;
  const int* __restrict__ rec_col;
  int nrec, nch;
  const float* __restrict__ resid;  // resid + (j-1)*nrec*nch (channel 0)
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

}  // namespace sgb
