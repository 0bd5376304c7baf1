// Argument checks shared by the extern "C" entry points (capi*.cu).
#pragma once
#include <cstdint>

#include "sgb_common.cuh"

namespace sgb {

// Device status word of the kernels (capi.cu).
int* status_ptr();

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

inline int check_grid(const sgb_grid* g) {
  if (g == nullptr) return SGB_ERR_ARG;
  if (g->nz <= 0 || g->nx <= 0 || g->nshots <= 0 || g->pitch < g->nx) return SGB_ERR_SHAPE;
  if (g->pitch % 4 != 0) return SGB_ERR_ALIGN;
  if (!(g->dt > 0.f) || !(g->h > 0.f)) return SGB_ERR_ARG;
  return SGB_OK;
}

inline int check_acq(const sgb_grid* g, const sgb_acquisition* q) {
  if (q == nullptr) return SGB_ERR_ARG;
  if (q->nt <= 0) return SGB_ERR_ARG;
  if (q->nsrc > 0 && (q->src_ptr == nullptr || q->src_z == nullptr || q->src_x == nullptr ||
                      q->src_wrow == nullptr || q->wavelet == nullptr))
    return SGB_ERR_ARG;
  if (q->records != nullptr && (q->rec_row_ptr == nullptr || q->rec_x == nullptr || q->rec_col == nullptr))
    return SGB_ERR_ARG;
  if (q->records != nullptr && q->nch <= 0) return SGB_ERR_ARG;
  (void)g;
  return SGB_OK;
}

}  // namespace sgb
