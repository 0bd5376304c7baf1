// Device kernels around the hot path for the plain FWI baseline: the L2
// misfit with its adjoint source (loss.py:409-421), illumination
// preconditioning and gradient masking (process.py:43-47, 115-118),
// separable Gaussian smoothing (signal.py:247-319, process.py:66-113) and
// the normalised steepest-descent update (optimizer.py:124-142).
#include <cuda_runtime.h>
#include <stdint.h>

#include "sgb_common.cuh"
#include "capi_util.cuh"

namespace sgb {
namespace {

int blocks_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

// resid = 2 (syn - obs); *loss += sum (syn - obs)^2 (double).
__global__ void l2_kernel(long long n, const float* syn, const float* obs, float* resid, double* loss) {
  double a = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float d = syn[i] - obs[i];
    if (resid != nullptr) resid[i] = 2.f * d;
    a += (double)d * (double)d;
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, a);
}

__global__ void precond_kernel(int nz, int nx, int pitch, const float* g, const float* illum, float eps,
                               const float* mask, float* out) {
  const long long n = (long long)nz * pitch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if ((int)(i % pitch) >= nx) {
      out[i] = 0.f;
      continue;
    }
    float v = g[i];
    if (mask != nullptr) v *= mask[i];
    if (illum != nullptr) v /= (illum[i] + eps);
    out[i] = v;
  }
}

// numpy 'reflect' index (mirror without repeating the edge).
__device__ __forceinline__ int reflect(int j, int n) {
  if (n == 1) return 0;
  const int period = 2 * (n - 1);
  j %= period;
  if (j < 0) j += period;
  return j < n ? j : period - j;
}

// One axis of the smoothing: out[i] = sum_{d=-r..r} w[d + r] in[reflect(i + d)].
__global__ void smooth_axis_kernel(int nz, int nx, int pitch, int axis, const float* w, int r, const float* in,
                                   float* out) {
  const long long n = (long long)nz * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / nx), x = (int)(i % nx);
    float a = 0.f;
    if (axis == 0) {
      for (int d = -r; d <= r; ++d) a = fmaf(w[d + r], in[(long long)reflect(z + d, nz) * pitch + x], a);
    } else {
      for (int d = -r; d <= r; ++d) a = fmaf(w[d + r], in[(long long)z * pitch + reflect(x + d, nx)], a);
    }
    out[(long long)z * pitch + x] = a;
  }
}

// max |clamp(g, lo, hi)| as the bits of a non-negative float.
__global__ void maxabs_kernel(long long n, const float* g, int clamp, float lo, float hi, unsigned* out) {
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v = g[i];
    if (clamp) v = fminf(fmaxf(v, lo), hi);
    m = fmaxf(m, fabsf(v));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void sd_kernel(long long n, float* p, const float* g, int clamp, float lo, float hi, float lr,
                          const unsigned* maxbits) {
  const float mx = __uint_as_float(*maxbits);
  const float alpha = mx > 0.f ? lr / mx : 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v = g[i];
    if (clamp) v = fminf(fmaxf(v, lo), hi);
    p[i] -= alpha * v;
  }
}

// Non-linear conjugate gradient (optimizer.py:144-224).  d = grad clamped to
// [lo, hi] when clamp.  sums: [0] |d|^2, [1] (d - gp) . d, [2] |gp|^2
// (float64 atomics), then beta (PR or FR; 0 when |gp| = 0), the direction
// dir = -d + beta dir, gp = d, max |dir| (bits in slot 3), and the update
// param += lr / max|dir| * dir.
__device__ __forceinline__ float clamp_to(float v, int clamp, float lo, float hi) {
  return clamp ? fminf(fmaxf(v, lo), hi) : v;
}

__global__ void ncg_dots_kernel(long long n, const float* g, const float* gp, int clamp, float lo, float hi,
                                double* sums) {
  double a = 0.0, b = 0.0, c = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double d = clamp_to(g[i], clamp, lo, hi), p = gp[i];
    a += d * d;
    b += (d - p) * d;
    c += p * p;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums, a);
    atomicAdd(sums + 1, b);
    atomicAdd(sums + 2, c);
  }
}

__global__ void ncg_dir_kernel(long long n, const float* g, int clamp, float lo, float hi, float* gp, float* dir,
                               int fletcher_reeves, const double* sums, unsigned* maxbits) {
  const double pn = sums[2];
  const float beta = pn == 0.0 ? 0.f : (float)((fletcher_reeves ? sums[0] : sums[1]) / pn);
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float d = clamp_to(g[i], clamp, lo, hi);
    const float v = -d + beta * dir[i];
    dir[i] = v;
    gp[i] = d;
    m = fmaxf(m, fabsf(v));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, __float_as_uint(m));
}

__global__ void ncg_update_kernel(long long n, float* p, const float* dir, float lr, const unsigned* maxbits) {
  const float mx = __uint_as_float(*maxbits);
  const float alpha = mx > 0.f ? lr / mx : 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] += alpha * dir[i];
}

// Zero-phase IIR filter of every trace (scipy.signal.filtfilt's default
// method as SeisSignal._filter_ calls it, signal.py:39-40): odd extension
// by padlen samples at both ends, a forward direct-form-II-transposed pass
// started from zi * first sample, a backward pass started from zi * its
// first sample, extension removed.  Records [nt][ntr] (trace fastest); one
// thread per trace; float64 state.  work: [nt + 2 padlen][ntr] doubles.
__global__ void filtfilt_kernel(int nt, int ntr, int nc, const double* b, const double* a, const double* zi,
                                int padlen, const float* in, float* out, double* work) {
  const int tr = blockIdx.x * blockDim.x + threadIdx.x;
  if (tr >= ntr) return;
  const int ne = nt + 2 * padlen;
  auto x_ext = [&](int i) -> double {  // odd extension
    if (i < padlen) return 2.0 * in[tr] - in[(long long)(padlen - i) * ntr + tr];
    if (i >= padlen + nt) {
      const int k = i - (padlen + nt);  // 0.. padlen-1
      return 2.0 * in[(long long)(nt - 1) * ntr + tr] - in[(long long)(nt - 2 - k) * ntr + tr];
    }
    return in[(long long)(i - padlen) * ntr + tr];
  };
  double z[16];
  const int m = nc - 1;  // state length
  double x0 = x_ext(0);
  for (int j = 0; j < m; ++j) z[j] = zi[j] * x0;
  for (int i = 0; i < ne; ++i) {
    const double x = x_ext(i);
    const double y = b[0] * x + (m > 0 ? z[0] : 0.0);
    for (int j = 0; j < m; ++j) z[j] = b[j + 1] * x - a[j + 1] * y + (j + 1 < m ? z[j + 1] : 0.0);
    work[(long long)i * ntr + tr] = y;
  }
  x0 = work[(long long)(ne - 1) * ntr + tr];
  for (int j = 0; j < m; ++j) z[j] = zi[j] * x0;
  for (int i = ne - 1; i >= 0; --i) {
    const double x = work[(long long)i * ntr + tr];
    const double y = b[0] * x + (m > 0 ? z[0] : 0.0);
    for (int j = 0; j < m; ++j) z[j] = b[j + 1] * x - a[j + 1] * y + (j + 1 < m ? z[j + 1] : 0.0);
    if (i >= padlen && i < padlen + nt) out[(long long)(i - padlen) * ntr + tr] = (float)y;
  }
}

}  // namespace
}  // namespace sgb

using namespace sgb;

extern "C" {

int sgb_l2_misfit(int64_t n, const float* syn, const float* obs, float* resid, double* loss, sgb_stream_t stream) {
  if (syn == nullptr || obs == nullptr || loss == nullptr) return SGB_ERR_ARG;
  if (n <= 0) return SGB_ERR_SHAPE;
  l2_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(n, syn, obs, resid, loss);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

int sgb_grad_precondition(int32_t nz, int32_t nx, int32_t pitch, const float* grad, const float* illum, float eps,
                          const float* mask, float* out, sgb_stream_t stream) {
  if (grad == nullptr || out == nullptr) return SGB_ERR_ARG;
  if (nz <= 0 || nx <= 0 || pitch < nx) return SGB_ERR_SHAPE;
  precond_kernel<<<blocks_for((long long)nz * pitch), 256, 0, (cudaStream_t)stream>>>(nz, nx, pitch, grad, illum,
                                                                                       eps, mask, out);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

int sgb_grad_smooth(int32_t nz, int32_t nx, int32_t pitch, const float* weights_z, int32_t radius_z,
                    const float* weights_x, int32_t radius_x, int32_t counts, float* grad, float* tmp,
                    sgb_stream_t stream) {
  if (grad == nullptr || tmp == nullptr || weights_z == nullptr || weights_x == nullptr) return SGB_ERR_ARG;
  if (nz <= 0 || nx <= 0 || pitch < nx || counts < 0 || radius_z < 0 || radius_x < 0) return SGB_ERR_SHAPE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = blocks_for((long long)nz * nx);
  for (int c = 0; c < counts; ++c) {
    smooth_axis_kernel<<<nb, 256, 0, s>>>(nz, nx, pitch, 0, weights_z, radius_z, grad, tmp);
    smooth_axis_kernel<<<nb, 256, 0, s>>>(nz, nx, pitch, 1, weights_x, radius_x, tmp, grad);
  }
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

int sgb_sd_step(int64_t n, float* param, const float* grad, float lr, int32_t clamp, float lo, float hi,
                uint32_t* scratch, sgb_stream_t stream) {
  if (param == nullptr || grad == nullptr || scratch == nullptr) return SGB_ERR_ARG;
  if (n <= 0) return SGB_ERR_SHAPE;
  cudaStream_t s = (cudaStream_t)stream;
  SGB_CUDA_CHECK(cudaMemsetAsync(scratch, 0, sizeof(uint32_t), s));
  maxabs_kernel<<<blocks_for(n), 256, 0, s>>>(n, grad, clamp, lo, hi, scratch);
  sd_kernel<<<blocks_for(n), 256, 0, s>>>(n, param, grad, clamp, lo, hi, lr, scratch);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

int sgb_ncg_step(int64_t n, float* param, const float* grad, float* prev_grad, float* direction, float lr,
                 int32_t beta_type, int32_t clamp, float lo, float hi, double* scratch, sgb_stream_t stream) {
  if (param == nullptr || grad == nullptr || prev_grad == nullptr || direction == nullptr || scratch == nullptr)
    return SGB_ERR_ARG;
  if (n <= 0) return SGB_ERR_SHAPE;
  if (beta_type != 0 && beta_type != 1) return SGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  SGB_CUDA_CHECK(cudaMemsetAsync(scratch, 0, 4 * sizeof(double), s));
  unsigned* maxbits = reinterpret_cast<unsigned*>(scratch + 3);
  ncg_dots_kernel<<<blocks_for(n), 256, 0, s>>>(n, grad, prev_grad, clamp, lo, hi, scratch);
  ncg_dir_kernel<<<blocks_for(n), 256, 0, s>>>(n, grad, clamp, lo, hi, prev_grad, direction, beta_type, scratch,
                                               maxbits);
  ncg_update_kernel<<<blocks_for(n), 256, 0, s>>>(n, param, direction, lr, maxbits);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

int sgb_filtfilt(int32_t nt, int32_t ntraces, int32_t ncoef, const double* b, const double* a, const double* zi,
                 int32_t padlen, const float* in, float* out, double* work, sgb_stream_t stream) {
  if (b == nullptr || a == nullptr || zi == nullptr || in == nullptr || out == nullptr || work == nullptr)
    return SGB_ERR_ARG;
  if (nt < 2 || ntraces <= 0 || ncoef < 1 || ncoef > 17 || padlen < 0 || padlen > nt - 1) return SGB_ERR_SHAPE;
  filtfilt_kernel<<<(ntraces + 127) / 128, 128, 0, (cudaStream_t)stream>>>(nt, ntraces, ncoef, b, a, zi, padlen,
                                                                            in, out, work);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

}  // extern "C"
