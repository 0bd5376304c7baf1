// Batched 2-D FFT operator of the viscoacoustic equation
// (seistorch/equations2d/vacoustic_habc.py:95-111):
//   K(x) = real(ifft2(|k| fft2(x))),  |k| = sqrt(fz^2 + fx^2),
// fz = fftfreq(nz, h), fx = fftfreq(nx, h) (cycles per metre).  |k| is real
// and even, so K maps real fields to real fields and two shots travel in one
// complex transform (shot 2p as the real part, 2p+1 as the imaginary part).
//
// Transforms: mixed-radix Stockham autosort (radices 4, 2, 3, 5, 7, then any
// remaining prime by its direct DFT), one stage per pass through shared
// memory, every thread computing outputs of the stage directly from the
// stage's R inputs and a twiddle table W_n^m (float2, built once per call in
// double precision).  Three launches: row transforms (with the input
// difference and optional pre-multiplier), column transforms forward, |k|,
// inverse (the whole column block stays in shared memory), and inverse row
// transforms with the 1/(nz nx) scale and the optional post-multiplier.
#include <cmath>

#include "sgb_common.cuh"

namespace sgb {
namespace {

constexpr int FFT_MAX_N = 8192;
constexpr int FFT_MAX_RAD = 24;

struct FftFactors {
  int n, nrad;
  int rad[FFT_MAX_RAD];
};

FftFactors factorize(int n) {
  FftFactors f;
  f.n = n;
  f.nrad = 0;
  for (int p : {4, 2, 3, 5, 7}) {
    while (n % p == 0 && f.nrad < FFT_MAX_RAD) {
      f.rad[f.nrad++] = p;
      n /= p;
    }
  }
  for (int p = 11; n > 1 && f.nrad < FFT_MAX_RAD; p += 2) {
    while (n % p == 0 && f.nrad < FFT_MAX_RAD) {
      f.rad[f.nrad++] = p;
      n /= p;
    }
  }
  if (n > 1) f.nrad = -1;  // cannot happen for n <= FFT_MAX_N
  return f;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// All stages of G length-n transforms laid out [n][G] in shared memory
// (a: input, b: scratch).  tw[m] = exp(-2 pi i m / n); inverse uses conj.
// Returns the buffer that holds the result.
__device__ float2* fft_stages(float2* a, float2* b, const float2* tw, const FftFactors& f, int G, bool inverse) {
  const int n = f.n;
  int Ns = 1;
  for (int s = 0; s < f.nrad; ++s) {
    const int R = f.rad[s], step = n / R, span = Ns * R, tws = n / span;
    for (int t = threadIdx.x; t < n * G; t += blockDim.x) {
      const int o = t / G, c = t - o * G;
      const int blk = o / span, rem = o - blk * span;
      const int j = blk * Ns + rem % Ns;
      float2 acc = make_float2(0.f, 0.f);
      int e = 0;  // r * rem mod span
      for (int r = 0; r < R; ++r) {
        const float2 x = a[(j + r * step) * G + c];
        const float2 w = tw[e * tws];
        const float2 p = inverse ? cmulc(x, w) : cmul(x, w);
        acc.x += p.x;
        acc.y += p.y;
        e += rem;
        if (e >= span) e -= span;
      }
      b[o * G + c] = acc;
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

struct KArgs {
  int nz, nx, pitch, nshots, npairs;
  long long sstride;
  float h;
  const float* __restrict__ pre;   // [nz][pitch] or null
  const float* __restrict__ u1;    // [nshots][nz][pitch]
  const float* __restrict__ u2;    // [nshots][nz][pitch] or null
  const float* __restrict__ post;  // [nz][pitch] or null
  float* __restrict__ out;         // [nshots][nz][pitch]
  float2* __restrict__ work;       // [npairs][nz][nx]
  const float2* __restrict__ twz;  // [nz]
  const float2* __restrict__ twx;  // [nx]
  FftFactors fz, fx;
};

__global__ void twiddle_kernel(float2* tw, int n) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)m / (double)n, &s, &c);
    tw[m] = make_float2((float)c, (float)s);
  }
}

// Forward row transforms of the packed pair (shot 2p + i shot 2p+1).
__global__ void __launch_bounds__(256) k_rows_fwd_kernel(const KArgs a) {
  extern __shared__ float2 sm[];
  const int n = a.nx;
  float2* A = sm;
  float2* B = sm + n;
  float2* T = sm + 2 * n;
  const int z = blockIdx.x, p = blockIdx.y;
  const int b0 = 2 * p, b1 = 2 * p + 1;
  const long long ro = (long long)z * a.pitch;
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    T[x] = a.twx[x];
    const float s = a.pre ? a.pre[ro + x] : 1.f;
    float re = a.u1[b0 * a.sstride + ro + x], im = 0.f;
    if (a.u2) re -= a.u2[b0 * a.sstride + ro + x];
    if (b1 < a.nshots) {
      im = a.u1[b1 * a.sstride + ro + x];
      if (a.u2) im -= a.u2[b1 * a.sstride + ro + x];
    }
    A[x] = make_float2(s * re, s * im);
  }
  __syncthreads();
  const float2* r = fft_stages(A, B, T, a.fx, 1, false);
  float2* w = a.work + ((long long)p * a.nz + z) * a.nx;
  for (int x = threadIdx.x; x < n; x += blockDim.x) w[x] = r[x];
}

// Column transforms of G adjacent columns: forward, times |k|, inverse.
__global__ void __launch_bounds__(256) k_cols_kernel(const KArgs a, int G) {
  extern __shared__ float2 sm[];
  const int n = a.nz;
  float2* A = sm;
  float2* B = sm + n * G;
  float2* T = sm + 2 * n * G;
  const int x0 = blockIdx.x * G, p = blockIdx.y;
  const int gw = min(G, a.nx - x0);
  float2* w = a.work + (long long)p * a.nz * a.nx;
  for (int i = threadIdx.x; i < n; i += blockDim.x) T[i] = a.twz[i];
  for (int t = threadIdx.x; t < n * G; t += blockDim.x) {
    const int z = t / G, c = t - z * G;
    A[t] = c < gw ? w[(long long)z * a.nx + x0 + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* r = fft_stages(A, B, T, a.fz, G, false);
  float2* o = (r == A) ? B : A;
  const float inv_nzh = 1.f / (a.nz * a.h), inv_nxh = 1.f / (a.nx * a.h);
  for (int t = threadIdx.x; t < n * G; t += blockDim.x) {
    const int z = t / G, c = t - z * G;
    const int xg = x0 + c;
    const int iz = z < (a.nz + 1) / 2 ? z : z - a.nz;    // fftfreq index
    const int ix = xg < (a.nx + 1) / 2 ? xg : xg - a.nx;
    const float fz = iz * inv_nzh, fx = ix * inv_nxh;
    const float kk = sqrtf(fz * fz + fx * fx);
    r[t] = make_float2(kk * r[t].x, kk * r[t].y);
  }
  __syncthreads();
  r = fft_stages(r, o, T, a.fz, G, true);
  for (int t = threadIdx.x; t < n * G; t += blockDim.x) {
    const int z = t / G, c = t - z * G;
    if (c < gw) w[(long long)z * a.nx + x0 + c] = r[t];
  }
}

// Inverse row transforms, 1/(nz nx), optional post-multiplier, unpacking.
__global__ void __launch_bounds__(256) k_rows_inv_kernel(const KArgs a) {
  extern __shared__ float2 sm[];
  const int n = a.nx;
  float2* A = sm;
  float2* B = sm + n;
  float2* T = sm + 2 * n;
  const int z = blockIdx.x, p = blockIdx.y;
  const float2* w = a.work + ((long long)p * a.nz + z) * a.nx;
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    T[x] = a.twx[x];
    A[x] = w[x];
  }
  __syncthreads();
  const float2* r = fft_stages(A, B, T, a.fx, 1, true);
  const float scale = 1.f / ((float)a.nz * (float)a.nx);
  const int b0 = 2 * p, b1 = 2 * p + 1;
  const long long ro = (long long)z * a.pitch;
  for (int x = threadIdx.x; x < a.pitch; x += blockDim.x) {
    float re = 0.f, im = 0.f;
    if (x < n) {
      const float s = scale * (a.post ? a.post[ro + x] : 1.f);
      re = s * r[x].x;
      im = s * r[x].y;
    }
    a.out[b0 * a.sstride + ro + x] = re;  // padding columns get 0
    if (b1 < a.nshots) a.out[b1 * a.sstride + ro + x] = im;
  }
}

}  // namespace

// Shared-memory bytes of the column launch for G columns.
static size_t cols_smem(int nz, int G) { return (size_t)(2 * nz * G + nz) * sizeof(float2); }

int vacoustic_kterm(const sgb_grid& g, const float* pre, const float* u1, const float* u2, const float* post,
                    float* out, float* work, float* tw, cudaStream_t s) {
  if (g.nz > FFT_MAX_N || g.nx > FFT_MAX_N) return SGB_ERR_UNSUPPORTED;
  KArgs a;
  a.nz = g.nz;
  a.nx = g.nx;
  a.pitch = g.pitch;
  a.nshots = g.nshots;
  a.npairs = (g.nshots + 1) / 2;
  a.sstride = (long long)g.nz * g.pitch;
  a.h = g.h;
  a.pre = pre;
  a.u1 = u1;
  a.u2 = u2;
  a.post = post;
  a.out = out;
  a.work = reinterpret_cast<float2*>(work);
  float2* twz = reinterpret_cast<float2*>(tw);
  float2* twx = twz + g.nz;
  a.twz = twz;
  a.twx = twx;
  a.fz = factorize(g.nz);
  a.fx = factorize(g.nx);
  if (a.fz.nrad < 0 || a.fx.nrad < 0) return SGB_ERR_UNSUPPORTED;
  twiddle_kernel<<<(g.nz + 255) / 256, 256, 0, s>>>(twz, g.nz);
  twiddle_kernel<<<(g.nx + 255) / 256, 256, 0, s>>>(twx, g.nx);
  const size_t row_smem = (size_t)3 * g.nx * sizeof(float2);
  int G = 16;
  while (G > 1 && cols_smem(g.nz, G) > 160 * 1024) G /= 2;
  const size_t col_smem = cols_smem(g.nz, G);
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(k_rows_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_rows_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess)
      return set_cuda_error(cudaGetLastError());
    attr_set = true;
  }
  if (row_smem > 200 * 1024 || col_smem > 200 * 1024) return SGB_ERR_UNSUPPORTED;
  k_rows_fwd_kernel<<<dim3((unsigned)g.nz, (unsigned)a.npairs), 256, row_smem, s>>>(a);
  k_cols_kernel<<<dim3((unsigned)((g.nx + G - 1) / G), (unsigned)a.npairs), 256, col_smem, s>>>(a, G);
  k_rows_inv_kernel<<<dim3((unsigned)g.nz, (unsigned)a.npairs), 256, row_smem, s>>>(a);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

}  // namespace sgb
