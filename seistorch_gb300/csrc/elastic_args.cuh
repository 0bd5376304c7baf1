// Kernel argument blocks of the elastic velocity-stress kernels (elastic.cu).
#pragma once

#include "sgb_common.cuh"

namespace sgb {

// Output columns of one warp strip.  A warp loads 128 columns
// [x0 - 4, x0 + 124) (32 lanes x float4) and writes the middle 120: lanes 0
// and 31 are the x halo of both stencil phases of the staggered step.
constexpr int EL_SW = 120;

struct ElCoef {
  const float* __restrict__ q;
  const float* __restrict__ e;
  const float* __restrict__ pa;
  const float* __restrict__ la;
  const float* __restrict__ ma;
  const float* __restrict__ bv;
};

// Point events of one step: sources (CSR by shot, one wavelet row per
// point) and receivers (CSR by shot and row).
struct ElPoints {
  const int* __restrict__ src_ptr;
  const int* __restrict__ src_z;
  const int* __restrict__ src_x;
  const int* __restrict__ src_wrow;
  const float* __restrict__ wavelet;
  const int* __restrict__ src_zr;
  int nt, t, src_fields;
  const int* __restrict__ rec_row_ptr;
  const int* __restrict__ rec_x;
  const int* __restrict__ rec_col;
  const int* __restrict__ rec_zr;
  int nrec, nch;
  int rec_fields[4];
};

// Forward step: out = step(in) + sources; records / ring / illumination.
struct ElFwdArgs {
  int nz, nx, pitch, nshots, nstrip, nband;
  long long sstride;
  const float* in[5];
  float* out[5];
  ElCoef c;
  ElPoints p;
  float* __restrict__ records;  // records + t * nrec * nch, or null
  float* __restrict__ illum;
  int illum_field;
  float* __restrict__ ring_out;  // [5][nshots][ring.size] of the new state, or null
  Ring ring;
  int* status;
};

// Reverse step i (mode 0): from s_{i+1} and the adjoint partial
// M^T a_{i+2}, writes s_i (reconstructed inside the box, ring from the
// store, 0 elsewhere), M^T a_{i+1} and accumulates the gradient terms inside
// the box.  Mode 1 (single-step VJP): s_in holds the step's output stresses,
// v_in its input velocities; no reconstruction, gradient everywhere.
struct ElBwdArgs {
  int nz, nx, pitch, nshots, nstrip, nband;
  long long sstride;
  const float* s_in[5];
  float* s_out[5];
  const float* v_in[2];
  const float* a_in[5];
  float* a_out[5];
  float* grad[3];  // lambda, mu, buoyancy terms [nshots][nz][pitch]
  ElCoef c;
  ElPoints p;
  const float* __restrict__ resid;    // dJ/d(records) + t * nrec * nch, or null
  const float* __restrict__ ring_in;  // ring of s_i [5][nshots][ring.size], or null (zeros)
  Ring ring;
  int* status;
};

}  // namespace sgb
