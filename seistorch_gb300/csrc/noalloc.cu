// Allocation-free variant of the acoustic adjoint (sgb_acoustic_backward_noalloc).
//
// For callers that cannot allocate device memory themselves -- e.g. a host
// application or plugin framework that owns all device memory and forbids
// cudaMalloc/cudaFree on its threads, or a processing loop that must not
// allocate once it runs.  The adjoint's scratch (three adjoint wavefields and
// the per-shot gradient accumulators) lives in one file-scope device array of
// fixed size that every GPU loading this library holds until the process
// exits.  The caller still passes the inputs (forward state, boundary store,
// residuals) and the output gradient.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "seistorch_gb300.h"

namespace sgb {
int set_cuda_error(cudaError_t e);
}

namespace {

// 8 Mi floats (32 MiB): room for 4 fields of nshots * nz * pitch floats up to
// 2,097,152 floats each (e.g. 8 shots of 228 x 356, or 2 shots of 500 x 1100).
constexpr size_t kScratchFloats = size_t(8) << 20;
__device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

// Host-side cache of the array's device address, one entry per device.  The
// array's name in host code is only a host-side stand-in; the address comes
// from cudaGetSymbolAddress with the device current.  Entries are atomic:
// host threads making their first call on a device at the same time each
// look the address up and store the same value.  cudaDeviceReset destroys
// the context the address belongs to, so a caller that resets a device must
// not call this entry point on that device again in the same process.
constexpr int kMaxDevices = 64;
std::atomic<float*> g_scratch_addr[kMaxDevices];

}  // namespace

extern "C" int sgb_acoustic_backward_noalloc(const sgb_grid* grid, const sgb_acoustic_model* model,
                                             const sgb_acquisition* acq, const sgb_bs_store* bs,
                                             float* const ubuf[3], int32_t ucur, int32_t uprev, float* grad_vp,
                                             sgb_stream_t stream) {
  if (grid == nullptr) return SGB_ERR_ARG;
  if (grid->nz <= 0 || grid->pitch <= 0 || grid->nshots <= 0) return SGB_ERR_SHAPE;
  const unsigned long long field =
      (unsigned long long)grid->nshots * (unsigned long long)grid->nz * (unsigned long long)grid->pitch;
  if (field > kScratchFloats / 4) return SGB_ERR_SCRATCH;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return sgb::set_cuda_error(e);
  if (dev < 0 || dev >= kMaxDevices) return SGB_ERR_ARG;
  float* base = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (base == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return sgb::set_cuda_error(e);
    base = static_cast<float*>(p);
    g_scratch_addr[dev].store(base, std::memory_order_release);
  }
  // field is a multiple of 4 floats (pitch % 4 == 0 is checked downstream),
  // so every sub-buffer keeps the 16-byte alignment the kernels need.
  float* const lbuf[3] = {base, base + field, base + 2 * field};
  float* grad_shot = base + 3 * field;
  // sgb_acoustic_backward zeroes the adjoint buffers and the accumulators
  // before its first step, so nothing left by an earlier call leaks in.
  return sgb_acoustic_backward(grid, model, acq, bs, ubuf, ucur, uprev, lbuf, grad_shot, grad_vp, stream);
}
