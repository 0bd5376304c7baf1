// extern "C" entry points of libseistorch_gb300 (see include/seistorch_gb300.h).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "sgb_common.cuh"
#include "acoustic_args.cuh"
#include "capi_util.cuh"
#include "tma.cuh"

namespace sgb {

static thread_local int g_last_cuda_error = 0;

int set_cuda_error(cudaError_t e) {
  g_last_cuda_error = (int)e;
  return SGB_ERR_CUDA;
}

// Device status word (bit flags set by kernels, e.g. DEV_ERR_CAPACITY).
__device__ int g_dev_status;

int* status_ptr() {
  static int* p = nullptr;
  static int dev = -1;
  int cur = 0;
  cudaGetDevice(&cur);
  if (p == nullptr || dev != cur) {
    if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_dev_status) != cudaSuccess) return nullptr;
    dev = cur;
  }
  return p;
}

FdWeights fd_weights(int order) {
  // Exact rationals of the order-2..8 central second-derivative weights
  // (the solution of the Taylor system in acoustic.py:5-30).
  FdWeights w;
  for (int i = 0; i < 5; ++i) w.c[i] = 0.f;
  double c[5] = {0, 0, 0, 0, 0};
  switch (order) {
    case 2: c[1] = 1.0; break;
    case 4: c[1] = 4.0 / 3.0; c[2] = -1.0 / 12.0; break;
    case 6: c[1] = 3.0 / 2.0; c[2] = -3.0 / 20.0; c[3] = 1.0 / 90.0; break;
    case 8: c[1] = 8.0 / 5.0; c[2] = -1.0 / 5.0; c[3] = 8.0 / 315.0; c[4] = -1.0 / 560.0; break;
  }
  double s = 0;
  for (int j = 1; j <= 4; ++j) s += c[j];
  w.c[0] = (float)(-4.0 * s);
  for (int j = 1; j <= 4; ++j) w.c[j] = (float)c[j];
  return w;
}

// kernels in acoustic.cu
cudaError_t launch_acoustic_fwd(int R, bool habc, int tz, const AcStepArgs& a, cudaStream_t s);
cudaError_t launch_acoustic_vjp(int R, const AcVjpArgs& a, cudaStream_t s);
cudaError_t launch_acoustic_coef(const sgb_grid& gr, const float* vp, const float* damp, int boundary,
                                 float* g, float* k, cudaStream_t s);
int acoustic_backward_impl(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                           const sgb_bs_store* bs, float* const ubuf[3], int32_t ucur, int32_t uprev,
                           float* const lbuf[3], float* grad_shot, float* grad_vp, bool born, cudaStream_t s,
                           const float* kz = nullptr, float* grad_shot2 = nullptr, float* grad_out2 = nullptr,
                           const float* rho_c = nullptr);
cudaError_t launch_acoustic_grad_reduce(const sgb_grid& gr, const float* grad_shot, const float* vp,
                                        const Ring& ring, float* grad_vp, cudaStream_t s);
int pick_tz(int nz, int nx, int nshots, int tz_max);
// streaming kernels in acoustic_stream.cu
cudaError_t launch_acoustic_fwd_stream(int R, const CUtensorMap* maps, const AcStreamArgs& a, cudaStream_t s,
                                       bool habc = false);
int habc_tile_rows(int R, int hb);
int vacoustic_kterm(const sgb_grid& g, const float* pre, const float* u1, const float* u2, const float* post,
                    float* out, float* work, float* tw, cudaStream_t s);

// Viscoacoustic extras of a forward loop: before each step the damping term
// extra = a_neg * K(U_n - U_{n-1}) is formed and added to the interior
// update (vacoustic_habc.py:86-111).
struct VacParams {
  const float* a_neg;
  float* extra;
  float* work;
  float* tw;
};
cudaError_t launch_acoustic_bwd_stream(int R, const CUtensorMap* maps, const AcBwdStreamArgs& a,
                                       cudaStream_t s);
int field_map(CUtensorMap* m, const float* p, int nz, int nx, int pitch, int nshots, int boxw, int rb,
              int bs = 1);
int coef_map(CUtensorMap* m, const float* coef, int nz, int nx, int pitch, int rb);
int plane_map(CUtensorMap* m, const float* p, int nz, int nx, int pitch, int boxw, int rb);
int fwd_tile_rows();
int fwd_tile_shots();
int bwd_tile_rows();
int stencil_box_width(int R);
int set_stream_config(int fwd, int bwd, int habc);
cudaError_t launch_habc_step_vjp(const sgb_grid& g, const sgb_acoustic_model& m, const sgb_habc_vjp_io& io,
                                 cudaStream_t s);
cudaError_t launch_habc_bwd(const sgb_grid& g, const sgb_acoustic_model& m, const sgb_acquisition& q,
                            const Ring& ring, const float* la1, const float* la2, float* lout, const float* uj,
                            const float* ujm1, float* uout, float* grad, const float* ring_in, int t_src,
                            const float* resid, const float* kz, float* grad2, const float* rho_c,
                            float* grad_rho, cudaStream_t s, const float* wpl = nullptr);
cudaError_t launch_habc_shares(const sgb_grid& g, const sgb_acoustic_model& m, float* planes, cudaStream_t s);

}  // namespace sgb

#include "acoustic_args.cuh"

using namespace sgb;

namespace {

// The bounded-wait path of every pipelined kernel, on its own: thread 0
// initialises an mbarrier that expects one arrival, arrives on it only when
// `arrive` is set, and then waits for its first phase for at most `polls`
// polls.  Without the arrival nothing ever completes the phase, so the wait
// runs out, sets DEV_ERR_TIMEOUT in the status word and the kernel returns
// normally.  No copy is in flight at any time.
__global__ void wait_probe_kernel(int* status, uint32_t polls, int arrive) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    if (arrive) mbar_arrive(&bar);
    mbar_wait_n(&bar, 0, status, polls);
  }
}

// Largest eigenvalue of -L for the order's cross stencil (per h^2): twice the
// maximum over the 1-D wavenumber of 2 sum_j c_j (1 - cos(j theta)).
double stencil_symbol_max_2d(int order) {
  const FdWeights w = fd_weights(order);
  double best = 0.0;
  for (int i = 0; i <= 4096; ++i) {
    const double th = M_PI * i / 4096.0;
    double s = 0.0;
    for (int j = 1; j <= 4; ++j) s += 2.0 * w.c[j] * (1.0 - std::cos(j * th));
    if (s > best) best = s;
  }
  return 2.0 * best;
}


int check_model(const sgb_grid* g, const sgb_acoustic_model* m) {
  if (m == nullptr || m->coef == nullptr) return SGB_ERR_ARG;
  if (m->order != 2 && m->order != 4 && m->order != 6 && m->order != 8) return SGB_ERR_UNSUPPORTED;
  if (m->boundary != 0 && m->boundary != 1) return SGB_ERR_ARG;
  if (!aligned16(m->coef)) return SGB_ERR_ALIGN;
  if (m->boundary == 1) {
    if (m->vp == nullptr || m->damp == nullptr) return SGB_ERR_ARG;
    // the one-way extrapolation reads two cells inward of each 50-cell strip;
    // width 0 is the unblended update of the reverse steps
    if (m->habc_width < 0 || m->habc_width + 2 > g->nx || m->habc_width + 2 > g->nz) return SGB_ERR_SHAPE;
  }
  return SGB_OK;
}

AcStepArgs base_step_args(const sgb_grid* g, const sgb_acoustic_model* m) {
  AcStepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nz = g->nz;
  a.nx = g->nx;
  a.pitch = g->pitch;
  a.nshots = g->nshots;
  a.ntx = (g->nx + TX - 1) / TX;
  a.sstride = (long long)g->nz * g->pitch;
  a.g = m->coef;
  a.k = m->coef + (long long)g->nz * g->pitch;
  a.w = fd_weights(m->order);
  a.vp = m->vp;
  a.hb = m->damp;
  a.lamf = 2.f * g->dt / g->h;
  a.muf = (g->dt * g->dt) / (g->h * g->h);
  a.hw = m->habc_width;
  a.multiple = m->multiple;
  a.ring.size = 0;
  a.ring.iz0 = a.ring.iz1 = a.ring.ix0 = a.ring.ix1 = 0;
  a.ring.rt = a.ring.rb = a.ring.rl = a.ring.rr = 0;
  a.status = status_ptr();
  return a;
}


int acoustic_forward_impl(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                          float* const buf[3], float* illum, const sgb_bs_store* bs, int32_t* cur_out,
                          int32_t* prev_out, const float* kz, cudaStream_t s, const float* rho_c = nullptr,
                          const VacParams* vac = nullptr);

// Arguments of the TMA tile pipeline from those of the tile kernel.
void fill_stream_args(AcStreamArgs& sa, const AcStepArgs& a, const sgb_acquisition* acq, int tzr) {
  sa.nz = a.nz; sa.nx = a.nx; sa.pitch = a.pitch; sa.nshots = a.nshots; sa.ntx = a.ntx;
  sa.zc = tzr;
  sa.nzc = (a.nz + tzr - 1) / tzr;
  sa.nseg = sa.nzc;
  sa.tpu = 1;
  sa.g = a.g;
  sa.k = a.k;
  sa.src_zr = acq->src_zr;
  sa.rec_zr = acq->rec_zr;
  sa.sstride = a.sstride;
  sa.w = a.w;
  sa.src_ptr = a.src_ptr; sa.src_z = a.src_z; sa.src_x = a.src_x; sa.src_wrow = a.src_wrow;
  sa.wavelet = a.wavelet; sa.nt = a.nt;
  sa.rec_row_ptr = a.rec_row_ptr; sa.rec_x = a.rec_x; sa.rec_col = a.rec_col;
  sa.nrec = a.nrec; sa.nch = a.nch;
  sa.ring = a.ring;
  sa.status = a.status;
}

void fill_stream_habc(AcStreamArgs& sa, const AcStepArgs& a) {
  sa.vp = a.vp;
  sa.hb = a.hb;
  sa.lamf = a.lamf;
  sa.muf = a.muf;
  sa.hw = a.hw;
  sa.multiple = a.multiple;
  sa.kz = a.kz;
  sa.rho_c = a.rho_c;
  sa.born_m = a.born_m;
  sa.born_out = a.born_out;
  sa.born_in = a.born_in;
}

}  // namespace

extern "C" {

const char* sgb_version(void) { return "seistorch_gb300 0.1.0 (sm_103a)"; }

const char* sgb_status_string(int s) {
  switch (s) {
    case SGB_OK: return "ok";
    case SGB_ERR_ARG: return "invalid argument";
    case SGB_ERR_SHAPE: return "inconsistent shape";
    case SGB_ERR_ALIGN: return "misaligned pointer or pitch";
    case SGB_ERR_CUDA: return "CUDA runtime error";
    case SGB_ERR_UNSUPPORTED: return "unsupported option";
    case SGB_ERR_NONFINITE: return "non-finite values in the records";
    case SGB_ERR_CAPACITY: return "too many sources inside one tile";
    case SGB_ERR_SCRATCH: return "problem larger than the fixed scratch of the allocation-free entry point";
    case SGB_ERR_CFL: return "CFL condition violated: max velocity * dt / h exceeds the scheme's stability limit";
  }
  return "unknown status";
}

int sgb_last_cuda_error(void) { return g_last_cuda_error; }

int sgb_cfl_check(int32_t scheme, int32_t order, float vmax, float dt, float h, float* courant_out,
                  float* limit_out) {
  if (!(dt > 0.f) || !(h > 0.f) || !(vmax >= 0.f) || !std::isfinite(vmax) || !std::isfinite(dt) ||
      !std::isfinite(h))
    return SGB_ERR_ARG;
  double limit;
  if (scheme == 0) {
    // u+ = 2u - u- + C^2 h^2 L(u) (leapfrog): stable while C^2 * max eig(-h^2 L) <= 4
    if (order != 2 && order != 4 && order != 6 && order != 8) return SGB_ERR_UNSUPPORTED;
    limit = 2.0 / std::sqrt(stencil_symbol_max_2d(order));
  } else if (scheme == 1) {
    // 2nd-order velocity-stress staggered grid: vp dt / h <= 1 / sqrt(2)
    if (order != 2) return SGB_ERR_UNSUPPORTED;
    limit = 1.0 / std::sqrt(2.0);
  } else {
    return SGB_ERR_ARG;
  }
  const double courant = (double)vmax * dt / h;
  if (courant_out != nullptr) *courant_out = (float)courant;
  if (limit_out != nullptr) *limit_out = (float)limit;
  return courant > limit ? SGB_ERR_CFL : SGB_OK;
}

int sgb_debug_wait_probe(uint32_t polls, int32_t arrive, sgb_stream_t stream) {
  int* st = status_ptr();
  if (st == nullptr) return SGB_ERR_CUDA;
  if (polls < 1 || polls > MBAR_SPIN_LIMIT) return SGB_ERR_ARG;
  wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(st, polls, arrive != 0);
  SGB_CUDA_CHECK(cudaGetLastError());
  return SGB_OK;
}

int sgb_device_status(int* out, int reset) {
  int* p = status_ptr();
  if (p == nullptr || out == nullptr) return SGB_ERR_ARG;
  SGB_CUDA_CHECK(cudaMemcpy(out, p, sizeof(int), cudaMemcpyDeviceToHost));
  if (reset) SGB_CUDA_CHECK(cudaMemset(p, 0, sizeof(int)));
  return SGB_OK;
}

int sgb_set_stream_config(int32_t fwd_cfg, int32_t bwd_cfg, int32_t habc_cfg) {
  return set_stream_config(fwd_cfg, bwd_cfg, habc_cfg) == 0 ? SGB_OK : SGB_ERR_ARG;
}

int sgb_ring_size(const sgb_grid* grid, int32_t iz0, int32_t iz1, int32_t ix0, int32_t ix1, int32_t ring,
                  int32_t* size_out) {
  if (int e = check_grid(grid)) return e;
  if (size_out == nullptr || ring < 1) return SGB_ERR_ARG;
  if (iz0 < 0 || ix0 < 0 || iz1 > grid->nz || ix1 > grid->nx || iz0 >= iz1 || ix0 >= ix1) return SGB_ERR_SHAPE;
  *size_out = make_ring(*grid, iz0, iz1, ix0, ix1, ring).size;
  return SGB_OK;
}

int sgb_acoustic_coefficients(const sgb_grid* grid, const float* vp, const float* damp, int32_t boundary,
                              float* coef_out, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (vp == nullptr || coef_out == nullptr) return SGB_ERR_ARG;
  if (boundary != 0 && boundary != 1) return SGB_ERR_ARG;
  SGB_CUDA_CHECK(launch_acoustic_coef(*grid, vp, damp, boundary, coef_out,
                                      coef_out + (long long)grid->nz * grid->pitch, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_acoustic_step(const sgb_grid* grid, const sgb_acoustic_model* model, const float* u, const float* um,
                      float* unext, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (u == nullptr || um == nullptr || unext == nullptr) return SGB_ERR_ARG;
  if (!aligned16(u) || !aligned16(um) || !aligned16(unext)) return SGB_ERR_ALIGN;
  if (unext == u || unext == um) return SGB_ERR_ARG;
  AcStepArgs a = base_step_args(grid, model);
  a.u = u;
  a.um = um;
  a.un = unext;
  const int tz = pick_tz(grid->nz, grid->nx, grid->nshots, 32);
  SGB_CUDA_CHECK(launch_acoustic_fwd(model->order / 2, model->boundary == 1, tz, a, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_acoustic_step_vjp(const sgb_grid* grid, const sgb_acoustic_model* model, const float* u,
                          const float* gy, const float* gh1, float* gu, float* gum, float* gvp_acc,
                          sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (model->vp == nullptr) return SGB_ERR_ARG;
  if (model->boundary == 1 && model->damp == nullptr) return SGB_ERR_ARG;
  if (u == nullptr || gy == nullptr || gu == nullptr || gum == nullptr || gvp_acc == nullptr) return SGB_ERR_ARG;
  if (!aligned16(u) || !aligned16(gy) || !aligned16(gu) || !aligned16(gum) || (gh1 && !aligned16(gh1)))
    return SGB_ERR_ALIGN;
  AcVjpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nz = grid->nz; a.nx = grid->nx; a.pitch = grid->pitch; a.nshots = grid->nshots;
  a.ntx = (grid->nx + TX - 1) / TX;
  a.sstride = (long long)grid->nz * grid->pitch;
  a.u = u; a.gy = gy; a.gh1 = gh1; a.gu = gu; a.gum = gum; a.gvp = gvp_acc;
  a.g = model->coef;
  a.k = model->coef + (long long)grid->nz * grid->pitch;
  a.vp = model->vp;
  a.w = fd_weights(model->order);
  SGB_CUDA_CHECK(launch_acoustic_vjp(model->order / 2, a, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_habc_step_vjp(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_habc_vjp_io* io,
                      sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (io == nullptr) return SGB_ERR_ARG;
  if (model->boundary != 1) return SGB_ERR_UNSUPPORTED;  // PML: sgb_acoustic_step_vjp
  if (io->kz != nullptr && io->rho_c != nullptr) return SGB_ERR_ARG;
  if ((io->kz != nullptr || io->rho_c != nullptr) && (model->order != 2 || io->born_m != nullptr))
    return SGB_ERR_UNSUPPORTED;
  const float* need[6] = {io->u, io->um, io->gy, io->gu, io->gum, io->gparam};
  for (const float* q : need) {
    if (q == nullptr) return SGB_ERR_ARG;
    if (!aligned16(q)) return SGB_ERR_ALIGN;
  }
  if (io->born_m != nullptr && (io->born_u == nullptr || io->born_gu == nullptr || io->born_gm == nullptr))
    return SGB_ERR_ARG;
  if (io->gu == io->gy || io->gum == io->gy || io->gu == io->gum) return SGB_ERR_ARG;
  SGB_CUDA_CHECK(launch_habc_step_vjp(*grid, *model, *io, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_acoustic_forward(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                         float* const buf[3], float* illum, const sgb_bs_store* bs, int32_t* cur_out,
                         int32_t* prev_out, sgb_stream_t stream) {
  return acoustic_forward_impl(grid, model, acq, buf, illum, bs, cur_out, prev_out, nullptr, (cudaStream_t)stream);
}

int sgb_vti_forward(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                    float* const buf[3], const sgb_bs_store* bs, int32_t* cur_out, int32_t* prev_out,
                    sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (model == nullptr || model->coef == nullptr) return SGB_ERR_ARG;
  if (model->boundary != 1 || model->order != 2) return SGB_ERR_UNSUPPORTED;  // vti_habc2: 2nd order, HABC
  return acoustic_forward_impl(grid, model, acq, buf, nullptr, bs, cur_out, prev_out,
                               model->coef + 2LL * grid->nz * grid->pitch, (cudaStream_t)stream);
}

int sgb_rho_forward(const sgb_grid* grid, const sgb_acoustic_model* model, const float* rho_c,
                    const sgb_acquisition* acq, float* const buf[3], const sgb_bs_store* bs, int32_t* cur_out,
                    int32_t* prev_out, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (model == nullptr || rho_c == nullptr) return SGB_ERR_ARG;
  if (model->boundary != 1 || model->order != 2) return SGB_ERR_UNSUPPORTED;  // acoustic_rho_habc: 2nd order, HABC
  if (!aligned16(rho_c)) return SGB_ERR_ALIGN;
  return acoustic_forward_impl(grid, model, acq, buf, nullptr, bs, cur_out, prev_out, nullptr, (cudaStream_t)stream,
                               rho_c);
}

int sgb_vacoustic_work_size(const sgb_grid* grid, int64_t* work_floats, int64_t* tw_floats) {
  if (int e = check_grid(grid)) return e;
  if (work_floats == nullptr || tw_floats == nullptr) return SGB_ERR_ARG;
  *work_floats = 2LL * ((grid->nshots + 1) / 2) * grid->nz * grid->nx;
  *tw_floats = 2LL * (grid->nz + grid->nx);
  return SGB_OK;
}

int sgb_vacoustic_kterm(const sgb_grid* grid, const float* pre, const float* u1, const float* u2, const float* post,
                        float* out, float* work, float* tw, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (u1 == nullptr || out == nullptr || work == nullptr || tw == nullptr) return SGB_ERR_ARG;
  if (out == u1 || out == u2) return SGB_ERR_ARG;
  return vacoustic_kterm(*grid, pre, u1, u2, post, out, work, tw, (cudaStream_t)stream);
}

int sgb_vacoustic_step(const sgb_grid* grid, const sgb_acoustic_model* model, const float* a_neg, const float* u,
                       const float* um, float* unext, float* extra, float* work, float* tw, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (model->boundary != 1) return SGB_ERR_UNSUPPORTED;
  if (a_neg == nullptr || u == nullptr || um == nullptr || unext == nullptr || extra == nullptr || work == nullptr ||
      tw == nullptr)
    return SGB_ERR_ARG;
  if (!aligned16(u) || !aligned16(um) || !aligned16(unext) || !aligned16(extra)) return SGB_ERR_ALIGN;
  if (unext == u || unext == um || extra == u || extra == um || extra == unext) return SGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (int e = vacoustic_kterm(*grid, nullptr, u, um, a_neg, extra, work, tw, s)) return e;
  AcStepArgs a = base_step_args(grid, model);
  a.u = u;
  a.um = um;
  a.un = unext;
  a.born_in = extra;
  const int tz = pick_tz(grid->nz, grid->nx, grid->nshots, 32);
  SGB_CUDA_CHECK(launch_acoustic_fwd(model->order / 2, true, tz, a, s));
  return SGB_OK;
}

int sgb_vacoustic_forward(const sgb_grid* grid, const sgb_acoustic_model* model, const float* a_neg,
                          const sgb_acquisition* acq, float* const buf[3], float* extra, float* work, float* tw,
                          int32_t* cur_out, int32_t* prev_out, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (model == nullptr || a_neg == nullptr || extra == nullptr || work == nullptr || tw == nullptr)
    return SGB_ERR_ARG;
  if (model->boundary != 1) return SGB_ERR_UNSUPPORTED;  // vacoustic_habc: HABC
  if (!aligned16(extra)) return SGB_ERR_ALIGN;
  const VacParams vac{a_neg, extra, work, tw};
  return acoustic_forward_impl(grid, model, acq, buf, nullptr, nullptr, cur_out, prev_out, nullptr,
                               (cudaStream_t)stream, nullptr, &vac);
}

}  // extern "C"

namespace {

int acoustic_forward_impl(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                          float* const buf[3], float* illum, const sgb_bs_store* bs, int32_t* cur_out,
                          int32_t* prev_out, const float* kz, cudaStream_t s, const float* rho_c,
                          const VacParams* vac) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (int e = check_acq(grid, acq)) return e;
  if (buf == nullptr || cur_out == nullptr || prev_out == nullptr) return SGB_ERR_ARG;
  for (int i = 0; i < 3; ++i) {
    if (buf[i] == nullptr) return SGB_ERR_ARG;
    if (!aligned16(buf[i])) return SGB_ERR_ALIGN;
  }
  if (acq->records != nullptr && acq->nch != 1) return SGB_ERR_UNSUPPORTED;
  AcStepArgs a = base_step_args(grid, model);
  a.kz = kz;
  a.rho_c = rho_c;
  a.src_ptr = acq->nsrc > 0 ? acq->src_ptr : nullptr;
  a.src_z = acq->src_z;
  a.src_x = acq->src_x;
  a.src_wrow = acq->src_wrow;
  a.wavelet = acq->wavelet;
  a.nt = acq->nt;
  a.rec_row_ptr = acq->rec_row_ptr;
  a.rec_x = acq->rec_x;
  a.rec_col = acq->rec_col;
  a.nrec = acq->nrec;
  a.nch = acq->nch;
  a.illum = illum;
  const long long plane = (long long)grid->nz * grid->pitch;
  const long long field = plane * grid->nshots;
  if (bs != nullptr) {
    if (bs->ring < 1 || bs->ring_store == nullptr) return SGB_ERR_ARG;
    if (bs->iz0 < 0 || bs->ix0 < 0 || bs->iz1 > grid->nz || bs->ix1 > grid->nx || bs->iz0 >= bs->iz1 ||
        bs->ix0 >= bs->ix1)
      return SGB_ERR_SHAPE;
    a.ring = make_ring(*grid, bs->iz0, bs->iz1, bs->ix0, bs->ix1, bs->ring);
    if (a.ring.size != bs->ring_size) return SGB_ERR_SHAPE;
    if (bs->ckpt_every > 0 && bs->ckpt_store == nullptr) return SGB_ERR_ARG;
  }
  const int R = model->order / 2;
  const bool habc = model->boundary == 1;
  // TMA tile pipeline for both boundaries (the HABC instantiation adds the
  // strip blend and the equation variants)
  CUtensorMap mu[3], mum[3];
  AcStreamArgs sa;
  std::memset(&sa, 0, sizeof(sa));
  const int tzr = habc ? habc_tile_rows(R, a.rho_c != nullptr ? 3 : (a.kz != nullptr ? 2 : 1)) : fwd_tile_rows();
  const int tsb = habc ? 1 : fwd_tile_shots();
  const int bw = stencil_box_width(R);
  for (int i = 0; i < 3; ++i)
    if (field_map(&mu[i], buf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, bw, tzr + 2 * R, tsb) ||
        field_map(&mum[i], buf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, TX, tzr, tsb))
      return SGB_ERR_CUDA;
  fill_stream_args(sa, a, acq, tzr);
  sa.illum = illum;
  if (habc) fill_stream_habc(sa, a);
  if ((a.src_ptr != nullptr && acq->src_zr == nullptr) || (acq->records != nullptr && acq->rec_zr == nullptr))
    return SGB_ERR_ARG;
  int cur = 0, prev = 1, nxt = 2;
  for (int t = 0; t < acq->nt; ++t) {
    sa.un = buf[nxt];
    sa.um = buf[prev];
    sa.u = buf[cur];
    sa.t = t;
    sa.records = acq->records ? acq->records + (long long)t * acq->nrec * acq->nch : nullptr;
    // the step saves the ring of its input U_t into slot t-1 (the adjoint
    // reads the rings of U_1 .. U_{nt-2})
    sa.ring_src = buf[cur];
    sa.ring_dst = (bs != nullptr && t >= 1) ? bs->ring_store + (long long)(t - 1) * grid->nshots * a.ring.size
                                            : nullptr;
    const CUtensorMap maps[2] = {mu[cur], mum[prev]};
    if (vac != nullptr) {
      if (int e = vacoustic_kterm(*grid, nullptr, buf[cur], buf[prev], vac->a_neg, vac->extra, vac->work, vac->tw, s))
        return e;
      sa.born_in = vac->extra;
    }
    SGB_CUDA_CHECK(launch_acoustic_fwd_stream(R, maps, sa, s, habc));
    if (bs != nullptr && bs->ckpt_every > 0 && (t + 1) % bs->ckpt_every == 0) {
      float* slot = bs->ckpt_store + (long long)((t + 1) / bs->ckpt_every - 1) * 2 * field;
      SGB_CUDA_CHECK(cudaMemcpyAsync(slot, buf[nxt], field * sizeof(float), cudaMemcpyDeviceToDevice, s));
      SGB_CUDA_CHECK(cudaMemcpyAsync(slot + field, buf[cur], field * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    prev = cur;
    cur = nxt;
    nxt = 3 - prev - cur;
  }
  *cur_out = cur;
  *prev_out = prev;
  return SGB_OK;
}

}  // namespace

extern "C" {

int sgb_born_forward(const sgb_grid* grid, const sgb_acoustic_model* model, const float* m,
                     const sgb_acquisition* acq, float* const pbuf[3], float* const sbuf[3], float* born_src,
                     const sgb_bs_store* bs, int32_t* cur_out, int32_t* prev_out, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (int e = check_acq(grid, acq)) return e;
  if (model->boundary != 1) return SGB_ERR_UNSUPPORTED;  // the reference's Born equation is HABC
  if (model->vp == nullptr || model->damp == nullptr) return SGB_ERR_ARG;
  if (m == nullptr || born_src == nullptr || pbuf == nullptr || sbuf == nullptr || cur_out == nullptr ||
      prev_out == nullptr)
    return SGB_ERR_ARG;
  if (!aligned16(m) || !aligned16(born_src)) return SGB_ERR_ALIGN;
  for (int i = 0; i < 3; ++i) {
    if (pbuf[i] == nullptr || sbuf[i] == nullptr) return SGB_ERR_ARG;
    if (!aligned16(pbuf[i]) || !aligned16(sbuf[i])) return SGB_ERR_ALIGN;
  }
  if (acq->records != nullptr && acq->nch != 1) return SGB_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  // background: sources, no receivers, writes m k L(p); scattered: receivers
  AcStepArgs ap = base_step_args(grid, model);
  ap.src_ptr = acq->nsrc > 0 ? acq->src_ptr : nullptr;
  ap.src_z = acq->src_z;
  ap.src_x = acq->src_x;
  ap.src_wrow = acq->src_wrow;
  ap.wavelet = acq->wavelet;
  ap.nt = acq->nt;
  ap.born_m = m;
  ap.born_out = born_src;
  AcStepArgs as = base_step_args(grid, model);
  as.nt = acq->nt;
  as.rec_row_ptr = acq->rec_row_ptr;
  as.rec_x = acq->rec_x;
  as.rec_col = acq->rec_col;
  as.nrec = acq->nrec;
  as.nch = acq->nch;
  as.born_in = born_src;
  const long long plane = (long long)grid->nz * grid->pitch;
  const long long field = plane * grid->nshots;
  Ring ring{};
  if (bs != nullptr) {  // boundary store of the background field
    if (bs->ring < 1 || bs->ring_store == nullptr) return SGB_ERR_ARG;
    if (bs->iz0 < 0 || bs->ix0 < 0 || bs->iz1 > grid->nz || bs->ix1 > grid->nx || bs->iz0 >= bs->iz1 ||
        bs->ix0 >= bs->ix1)
      return SGB_ERR_SHAPE;
    ring = make_ring(*grid, bs->iz0, bs->iz1, bs->ix0, bs->ix1, bs->ring);
    if (ring.size != bs->ring_size) return SGB_ERR_SHAPE;
    if (bs->ckpt_every > 0 && bs->ckpt_store == nullptr) return SGB_ERR_ARG;
  }
  const int R = model->order / 2;
  ap.ring = ring;
  const int tzr = habc_tile_rows(R, 1);
  const int bw = stencil_box_width(R);
  CUtensorMap pu[3], pum[3], su3[3], sum3[3];
  for (int i = 0; i < 3; ++i)
    if (field_map(&pu[i], pbuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, bw, tzr + 2 * R) ||
        field_map(&pum[i], pbuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, TX, tzr) ||
        field_map(&su3[i], sbuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, bw, tzr + 2 * R) ||
        field_map(&sum3[i], sbuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, TX, tzr))
      return SGB_ERR_CUDA;
  AcStreamArgs sp, ss;
  std::memset(&sp, 0, sizeof(sp));
  std::memset(&ss, 0, sizeof(ss));
  fill_stream_args(sp, ap, acq, tzr);
  fill_stream_habc(sp, ap);
  fill_stream_args(ss, as, acq, tzr);
  fill_stream_habc(ss, as);
  if ((ap.src_ptr != nullptr && acq->src_zr == nullptr) || (acq->records != nullptr && acq->rec_zr == nullptr))
    return SGB_ERR_ARG;
  for (int i = 0; i < 3; ++i) {
    SGB_CUDA_CHECK(cudaMemsetAsync(pbuf[i], 0, field * sizeof(float), s));
    SGB_CUDA_CHECK(cudaMemsetAsync(sbuf[i], 0, field * sizeof(float), s));
  }
  int cur = 0, prev = 1, nxt = 2;
  for (int t = 0; t < acq->nt; ++t) {
    sp.u = pbuf[cur];
    sp.um = pbuf[prev];
    sp.un = pbuf[nxt];
    sp.t = t;
    // the background step saves the ring of its input U_t into slot t-1
    sp.ring_src = pbuf[cur];
    sp.ring_dst = (bs != nullptr && t >= 1) ? bs->ring_store + (long long)(t - 1) * grid->nshots * ring.size : nullptr;
    const CUtensorMap mp[2] = {pu[cur], pum[prev]};
    SGB_CUDA_CHECK(launch_acoustic_fwd_stream(R, mp, sp, s, true));
    ss.u = sbuf[cur];
    ss.um = sbuf[prev];
    ss.un = sbuf[nxt];
    ss.t = t;
    ss.records = acq->records ? acq->records + (long long)t * acq->nrec * acq->nch : nullptr;
    const CUtensorMap ms[2] = {su3[cur], sum3[prev]};
    SGB_CUDA_CHECK(launch_acoustic_fwd_stream(R, ms, ss, s, true));
    if (bs != nullptr && bs->ckpt_every > 0 && (t + 1) % bs->ckpt_every == 0) {
      float* slot = bs->ckpt_store + (long long)((t + 1) / bs->ckpt_every - 1) * 2 * field;
      SGB_CUDA_CHECK(cudaMemcpyAsync(slot, pbuf[nxt], field * sizeof(float), cudaMemcpyDeviceToDevice, s));
      SGB_CUDA_CHECK(cudaMemcpyAsync(slot + field, pbuf[cur], field * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    prev = cur;
    cur = nxt;
    nxt = 3 - prev - cur;
  }
  *cur_out = cur;
  *prev_out = prev;
  return SGB_OK;
}

int sgb_born_step(const sgb_grid* grid, const sgb_acoustic_model* model, const float* m, const float* p,
                  const float* pm, const float* sc, const float* scm, float* pnext, float* snext, float* born_src,
                  sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (model->boundary != 1) return SGB_ERR_UNSUPPORTED;
  if (model->vp == nullptr || model->damp == nullptr) return SGB_ERR_ARG;
  const float* in[6] = {m, p, pm, sc, scm, born_src};
  for (const float* q : in) {
    if (q == nullptr) return SGB_ERR_ARG;
    if (!aligned16(q)) return SGB_ERR_ALIGN;
  }
  if (pnext == nullptr || snext == nullptr) return SGB_ERR_ARG;
  if (!aligned16(pnext) || !aligned16(snext)) return SGB_ERR_ALIGN;
  if (pnext == p || pnext == pm || snext == sc || snext == scm) return SGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int tz = pick_tz(grid->nz, grid->nx, grid->nshots, 32);
  AcStepArgs a = base_step_args(grid, model);
  a.u = p;
  a.um = pm;
  a.un = pnext;
  a.born_m = m;
  a.born_out = born_src;
  SGB_CUDA_CHECK(launch_acoustic_fwd(model->order / 2, true, tz, a, s));
  AcStepArgs b = base_step_args(grid, model);
  b.u = sc;
  b.um = scm;
  b.un = snext;
  b.born_in = born_src;
  SGB_CUDA_CHECK(launch_acoustic_fwd(model->order / 2, true, tz, b, s));
  return SGB_OK;
}

int sgb_vti_backward(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                     const sgb_bs_store* bs, float* const ubuf[3], int32_t ucur, int32_t uprev, float* const lbuf[3],
                     float* grad_shot_x, float* grad_shot_z, float* grad_x, float* grad_z, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (model == nullptr || model->coef == nullptr) return SGB_ERR_ARG;
  if (model->boundary != 1 || model->order != 2) return SGB_ERR_UNSUPPORTED;
  if (grad_shot_z == nullptr || grad_z == nullptr) return SGB_ERR_ARG;
  if (!aligned16(grad_shot_z)) return SGB_ERR_ALIGN;
  return sgb::acoustic_backward_impl(grid, model, acq, bs, ubuf, ucur, uprev, lbuf, grad_shot_x, grad_x, false,
                                     (cudaStream_t)stream, model->coef + 2LL * grid->nz * grid->pitch, grad_shot_z,
                                     grad_z);
}

int sgb_rho_backward(const sgb_grid* grid, const sgb_acoustic_model* model, const float* rho_c,
                     const sgb_acquisition* acq, const sgb_bs_store* bs, float* const ubuf[3], int32_t ucur,
                     int32_t uprev, float* const lbuf[3], float* grad_shot5, float* grad5, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (model == nullptr || rho_c == nullptr) return SGB_ERR_ARG;
  if (model->boundary != 1 || model->order != 2) return SGB_ERR_UNSUPPORTED;
  if (!aligned16(rho_c)) return SGB_ERR_ALIGN;
  return sgb::acoustic_backward_impl(grid, model, acq, bs, ubuf, ucur, uprev, lbuf, grad_shot5, grad5, false,
                                     (cudaStream_t)stream, nullptr, nullptr, nullptr, rho_c);
}

int sgb_rho_step(const sgb_grid* grid, const sgb_acoustic_model* model, const float* rho_c, const float* u,
                 const float* um, float* unext, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (model->boundary != 1 || model->order != 2) return SGB_ERR_UNSUPPORTED;
  if (model->vp == nullptr || model->damp == nullptr || rho_c == nullptr) return SGB_ERR_ARG;
  if (u == nullptr || um == nullptr || unext == nullptr) return SGB_ERR_ARG;
  if (!aligned16(u) || !aligned16(um) || !aligned16(unext) || !aligned16(rho_c)) return SGB_ERR_ALIGN;
  if (unext == u || unext == um) return SGB_ERR_ARG;
  AcStepArgs a = base_step_args(grid, model);
  a.u = u;
  a.um = um;
  a.un = unext;
  a.rho_c = rho_c;
  const int tz = pick_tz(grid->nz, grid->nx, grid->nshots, 32);
  SGB_CUDA_CHECK(launch_acoustic_fwd(1, true, tz, a, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_vti_step(const sgb_grid* grid, const sgb_acoustic_model* model, const float* u, const float* um,
                 float* unext, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (model->boundary != 1 || model->order != 2) return SGB_ERR_UNSUPPORTED;
  if (model->vp == nullptr || model->damp == nullptr) return SGB_ERR_ARG;
  if (u == nullptr || um == nullptr || unext == nullptr) return SGB_ERR_ARG;
  if (!aligned16(u) || !aligned16(um) || !aligned16(unext)) return SGB_ERR_ALIGN;
  if (unext == u || unext == um) return SGB_ERR_ARG;
  AcStepArgs a = base_step_args(grid, model);
  a.u = u;
  a.um = um;
  a.un = unext;
  a.kz = model->coef + 2LL * grid->nz * grid->pitch;
  const int tz = pick_tz(grid->nz, grid->nx, grid->nshots, 32);
  SGB_CUDA_CHECK(launch_acoustic_fwd(1, true, tz, a, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_born_backward(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                      const sgb_bs_store* bs, float* const pbuf[3], int32_t pcur, int32_t pprev, float* const lbuf[3],
                      float* grad_shot, float* grad_m, sgb_stream_t stream) {
  return sgb::acoustic_backward_impl(grid, model, acq, bs, pbuf, pcur, pprev, lbuf, grad_shot, grad_m, true,
                                     (cudaStream_t)stream);
}

int sgb_acoustic_backward(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                          const sgb_bs_store* bs, float* const ubuf[3], int32_t ucur, int32_t uprev,
                          float* const lbuf[3], float* grad_shot, float* grad_vp, sgb_stream_t stream) {
  return sgb::acoustic_backward_impl(grid, model, acq, bs, ubuf, ucur, uprev, lbuf, grad_shot, grad_vp, false,
                                     (cudaStream_t)stream);
}

}  // extern "C"

namespace sgb {

// The reverse loop of sgb_acoustic_backward; with `born` (HABC only) the
// adjoint runs the scattered field's recursion against the background's
// reconstruction and the reduction returns sum La k L(U) (dJ/dm of Born
// modelling) instead of (2/vp) times it (dJ/dvp).
int acoustic_backward_impl(const sgb_grid* grid, const sgb_acoustic_model* model, const sgb_acquisition* acq,
                           const sgb_bs_store* bs, float* const ubuf[3], int32_t ucur, int32_t uprev,
                           float* const lbuf[3], float* grad_shot, float* grad_vp, bool born, cudaStream_t s,
                           const float* kz, float* grad_shot2, float* grad_out2, const float* rho_c) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_model(grid, model)) return e;
  if (int e = check_acq(grid, acq)) return e;
  if (model->vp == nullptr) return SGB_ERR_ARG;
  if (model->boundary == 1 && model->damp == nullptr) return SGB_ERR_ARG;
  if (bs == nullptr || bs->ring_store == nullptr || ubuf == nullptr || lbuf == nullptr || grad_shot == nullptr ||
      grad_vp == nullptr)
    return SGB_ERR_ARG;
  if (ucur < 0 || ucur > 2 || uprev < 0 || uprev > 2 || ucur == uprev) return SGB_ERR_ARG;
  for (int i = 0; i < 3; ++i) {
    if (ubuf[i] == nullptr || lbuf[i] == nullptr) return SGB_ERR_ARG;
    if (!aligned16(ubuf[i]) || !aligned16(lbuf[i])) return SGB_ERR_ALIGN;
  }
  if (!aligned16(grad_shot)) return SGB_ERR_ALIGN;
  if (acq->records != nullptr && acq->nch != 1) return SGB_ERR_UNSUPPORTED;
  if ((born || kz != nullptr || rho_c != nullptr) && model->boundary != 1) return SGB_ERR_UNSUPPORTED;
  if (kz != nullptr && (grad_shot2 == nullptr || grad_out2 == nullptr)) return SGB_ERR_ARG;
  // dJ/dvp = (2/vp) sum La k L(U); Born (dJ/dm), VTI (dJ/dk, dJ/dkz) and
  // variable density (five coefficient gradients) keep the plain sums.  With
  // rho_c, grad_shot holds five fields and grad_vp five planes.
  const float* gscale = (born || kz != nullptr || rho_c != nullptr) ? nullptr : model->vp;
  const int ngrad = rho_c != nullptr ? 5 : 1;
  const long long plane = (long long)grid->nz * grid->pitch;
  const long long field = plane * grid->nshots;
  const Ring ring = make_ring(*grid, bs->iz0, bs->iz1, bs->ix0, bs->ix1, bs->ring);
  if (ring.size != bs->ring_size) return SGB_ERR_SHAPE;
  for (int i = 0; i < 3; ++i) SGB_CUDA_CHECK(cudaMemsetAsync(lbuf[i], 0, field * sizeof(float), s));
  // the adjoints accumulate every shot into plane 0 of each gradient field
  for (int q = 0; q < ngrad; ++q) SGB_CUDA_CHECK(cudaMemsetAsync(grad_shot + q * field, 0, plane * sizeof(float), s));
  if (grad_shot2 != nullptr) SGB_CUDA_CHECK(cudaMemsetAsync(grad_shot2, 0, plane * sizeof(float), s));
  const int R = model->order / 2;
  const int nt = acq->nt;
  const int K = bs->ckpt_every;
  const int nslots = K > 0 ? nt / K : 0;
  if (model->boundary == 1) {
    // HABC: tiled reverse-step kernel (habc_bwd.cu), same buffer rotation
    if ((acq->nsrc > 0 && acq->src_ptr == nullptr)) return SGB_ERR_ARG;
    int uj = ucur, ujm1 = uprev, ufree = 3 - ucur - uprev;
    int l1 = 0, l2 = 1, lfree = 2;
    // the cells' static interior / side shares, once for the whole reverse loop
    const float* wpl = nullptr;
    if (bs->habc_planes != nullptr) {
      if (!aligned16(bs->habc_planes)) return SGB_ERR_ALIGN;
      SGB_CUDA_CHECK(launch_habc_shares(*grid, *model, bs->habc_planes, s));
      wpl = bs->habc_planes;
    }
    for (int j = nt; j >= 2; --j) {
      const int n = j - 1;
      const bool ck = K > 0 && n % K == 0 && n / K >= 1 && n / K <= nslots;
      if (ck && n < nt) {
        const float* slot = bs->ckpt_store + (long long)(n / K - 1) * 2 * field;
        SGB_CUDA_CHECK(cudaMemcpyAsync(ubuf[ujm1], slot, field * sizeof(float), cudaMemcpyDeviceToDevice, s));
      }
      const float* ring_in = j >= 3 ? bs->ring_store + (long long)(j - 3) * grid->nshots * ring.size : nullptr;
      const float* resid = acq->records ? acq->records + (long long)(j - 1) * acq->nrec * acq->nch : nullptr;
      SGB_CUDA_CHECK(launch_habc_bwd(*grid, *model, *acq, ring, lbuf[l1], lbuf[l2], lbuf[lfree], ubuf[uj],
                                     ubuf[ujm1], j >= 3 ? ubuf[ufree] : nullptr, grad_shot, ring_in, j - 1, resid,
                                     kz, grad_shot2, rho_c, rho_c != nullptr ? grad_shot : nullptr, s, wpl));
      if (ck && j >= 3) {
        const float* slot = bs->ckpt_store + (long long)(n / K - 1) * 2 * field;
        SGB_CUDA_CHECK(
            cudaMemcpyAsync(ubuf[ufree], slot + field, field * sizeof(float), cudaMemcpyDeviceToDevice, s));
      }
      const int old_uj = uj;
      uj = ujm1;
      ujm1 = ufree;
      ufree = old_uj;
      const int old_l2 = l2;
      l2 = l1;
      l1 = lfree;
      lfree = old_l2;
    }
    // the buoyancy planes also carry terms on the box's one-cell rim
    Ring rim = ring;
    rim.iz0 = ring.iz0 > 0 ? ring.iz0 - 1 : 0;
    rim.ix0 = ring.ix0 > 0 ? ring.ix0 - 1 : 0;
    rim.iz1 = ring.iz1 < grid->nz ? ring.iz1 + 1 : grid->nz;
    rim.ix1 = ring.ix1 < grid->nx ? ring.ix1 + 1 : grid->nx;
    // every shot's terms went into plane 0 of each gradient field
    sgb_grid one = *grid;
    one.nshots = 1;
    for (int q = 0; q < ngrad; ++q)
      SGB_CUDA_CHECK(launch_acoustic_grad_reduce(one, grad_shot + q * field, gscale, q == 0 ? ring : rim,
                                                 grad_vp + q * plane, s));
    if (kz != nullptr) SGB_CUDA_CHECK(launch_acoustic_grad_reduce(one, grad_shot2, nullptr, ring, grad_out2, s));
    return SGB_OK;
  }
  // tensor maps: haloed stencil boxes (136 x (TZ+2R)) and point boxes
  // (128 x TZ) of every rotating buffer; lbuf carries nu = k * Lambda
  const int tzr = bwd_tile_rows();
  const int bw = stencil_box_width(R);
  CUtensorMap uf[3], nf[3], up[3], np[3], cm;
  for (int i = 0; i < 3; ++i) {
    if (field_map(&uf[i], ubuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, bw, tzr + 2 * R) ||
        field_map(&nf[i], lbuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, bw, tzr + 2 * R) ||
        field_map(&up[i], ubuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, TX, tzr) ||
        field_map(&np[i], lbuf[i], grid->nz, grid->nx, grid->pitch, grid->nshots, TX, tzr))
      return SGB_ERR_CUDA;
  }
  if (coef_map(&cm, model->coef, grid->nz, grid->nx, grid->pitch, tzr)) return SGB_ERR_CUDA;
  if ((acq->nsrc > 0 && acq->src_zr == nullptr) || (acq->records != nullptr && acq->rec_zr == nullptr))
    return SGB_ERR_ARG;
  AcBwdStreamArgs sb;
  std::memset(&sb, 0, sizeof(sb));
  sb.nz = grid->nz; sb.nx = grid->nx; sb.pitch = grid->pitch; sb.nshots = grid->nshots;
  sb.ntx = (grid->nx + TX - 1) / TX;
  sb.zc = tzr;
  sb.nzc = (grid->nz + tzr - 1) / tzr;
  sb.nseg = sb.nzc;
  sb.tpu = 1;
  sb.g = model->coef;
  sb.k = model->coef + plane;
  sb.src_zr = acq->src_zr;
  sb.rec_zr = acq->rec_zr;
  sb.sstride = plane;
  sb.grad_shot = grad_shot;
  sb.w = fd_weights(model->order);
  sb.ring = ring;
  sb.src_ptr = acq->nsrc > 0 ? acq->src_ptr : nullptr;
  sb.src_z = acq->src_z; sb.src_x = acq->src_x; sb.src_wrow = acq->src_wrow; sb.wavelet = acq->wavelet;
  sb.nt = acq->nt;
  sb.rec_row_ptr = acq->rec_row_ptr; sb.rec_x = acq->rec_x; sb.rec_col = acq->rec_col;
  sb.nrec = acq->nrec; sb.nch = acq->nch;
  sb.status = status_ptr();
  int uj = ucur, ujm1 = uprev, ufree = 3 - ucur - uprev;
  int l1 = 0, l2 = 1, lfree = 2;
  for (int j = nt; j >= 2; --j) {
    const int n = j - 1;
    const bool ck = K > 0 && n % K == 0 && n / K >= 1 && n / K <= nslots;
    if (ck && n < nt) {
      const float* slot = bs->ckpt_store + (long long)(n / K - 1) * 2 * field;
      SGB_CUDA_CHECK(cudaMemcpyAsync(ubuf[ujm1], slot, field * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    sb.lout = lbuf[lfree];
    sb.uout = ubuf[ufree];
    sb.unext = ubuf[uj];
    sb.n2 = lbuf[l2];
    sb.do_recon = j >= 3;
    sb.t_src = j - 1;
    sb.resid = acq->records ? acq->records + (long long)(j - 1) * acq->nrec * acq->nch : nullptr;
    const CUtensorMap maps[5] = {uf[ujm1], nf[l1], up[uj], np[l2], cm};
    sb.ring_in = j >= 3 ? bs->ring_store + (long long)(j - 3) * grid->nshots * ring.size : nullptr;
    SGB_CUDA_CHECK(launch_acoustic_bwd_stream(R, maps, sb, s));
    if (ck && j >= 3) {
      const float* slot = bs->ckpt_store + (long long)(n / K - 1) * 2 * field;
      SGB_CUDA_CHECK(cudaMemcpyAsync(ubuf[ufree], slot + field, field * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    const int old_uj = uj;
    uj = ujm1;
    ujm1 = ufree;
    ufree = old_uj;
    const int old_l2 = l2;
    l2 = l1;
    l1 = lfree;
    lfree = old_l2;
  }
  // every shot's gradient term went into plane 0 of grad_shot
  sgb_grid one = *grid;
  one.nshots = 1;
  SGB_CUDA_CHECK(launch_acoustic_grad_reduce(one, grad_shot, gscale, ring, grad_vp, s));
  return SGB_OK;
}

}  // namespace sgb
