// extern "C" entry points of the elastic velocity-stress path
// (include/seistorch_gb300.h; kernels in elastic.cu).
#include <cstring>

#include "sgb_common.cuh"
#include "capi_util.cuh"
#include "elastic_args.cuh"

namespace sgb {
void elastic_strip_geometry(int nz, int nx, int* nstrip, int* nband);
cudaError_t launch_elastic_fwd(const ElFwdArgs& a, cudaStream_t s);
cudaError_t launch_elastic_bwd(const ElBwdArgs& a, int mode, cudaStream_t s);
cudaError_t launch_elastic_coef(const sgb_grid& g, const float* vp, const float* vs, const float* rho,
                                const float* d, float* coef, cudaStream_t s);
cudaError_t launch_elastic_grad(const sgb_grid& g, const float* coef, const float* const gs[3], const float* vp,
                                const float* vs, const float* rho, int boxed, int iz0, int iz1, int ix0, int ix1,
                                float* const out[3], cudaStream_t s);
}  // namespace sgb

using namespace sgb;

namespace {

int check_emodel(const sgb_elastic_model* m) {
  if (m == nullptr || m->coef == nullptr) return SGB_ERR_ARG;
  if (!aligned16(m->coef)) return SGB_ERR_ALIGN;
  return SGB_OK;
}

int check_fields(const float* const* f, int n) {
  if (f == nullptr) return SGB_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    if (f[i] == nullptr) return SGB_ERR_ARG;
    if (!aligned16(f[i])) return SGB_ERR_ALIGN;
  }
  return SGB_OK;
}

int check_io(const sgb_elastic_io* io, const sgb_acquisition* q) {
  if (io == nullptr) return SGB_ERR_ARG;
  if (io->src_fields < 0 || io->src_fields >= (1 << SGB_ELASTIC_FIELDS)) return SGB_ERR_ARG;
  if (io->illum_field < 0 || io->illum_field >= SGB_ELASTIC_FIELDS) return SGB_ERR_ARG;
  if (q != nullptr && q->records != nullptr) {
    if (q->nch < 1 || q->nch > 4) return SGB_ERR_UNSUPPORTED;
    for (int c = 0; c < q->nch; ++c)
      if (io->rec_fields[c] < 0 || io->rec_fields[c] >= SGB_ELASTIC_FIELDS) return SGB_ERR_ARG;
  }
  return SGB_OK;
}

ElCoef coef_planes(const sgb_grid* g, const sgb_elastic_model* m) {
  const long long n = (long long)g->nz * g->pitch;
  ElCoef c;
  c.q = m->coef;
  c.e = m->coef + n;
  c.pa = m->coef + 2 * n;
  c.la = m->coef + 3 * n;
  c.ma = m->coef + 4 * n;
  c.bv = m->coef + 5 * n;
  return c;
}

void fill_points(ElPoints& p, const sgb_acquisition* q, const sgb_elastic_io* io) {
  std::memset(&p, 0, sizeof(p));
  if (q == nullptr) return;
  p.src_ptr = q->nsrc > 0 ? q->src_ptr : nullptr;
  p.src_z = q->src_z;
  p.src_x = q->src_x;
  p.src_wrow = q->src_wrow;
  p.wavelet = q->wavelet;
  p.src_zr = q->src_zr;
  p.nt = q->nt;
  p.src_fields = io ? io->src_fields : 0;
  p.rec_row_ptr = q->rec_row_ptr;
  p.rec_x = q->rec_x;
  p.rec_col = q->rec_col;
  p.rec_zr = q->rec_zr;
  p.nrec = q->nrec;
  p.nch = q->records ? q->nch : 0;
  for (int c = 0; c < 4; ++c) p.rec_fields[c] = io ? io->rec_fields[c] : 0;
}

template <class Args>
void fill_geometry(Args& a, const sgb_grid* g) {
  a.nz = g->nz;
  a.nx = g->nx;
  a.pitch = g->pitch;
  a.nshots = g->nshots;
  a.sstride = (long long)g->nz * g->pitch;
  elastic_strip_geometry(g->nz, g->nx, &a.nstrip, &a.nband);
}

int check_bs(const sgb_grid* g, const sgb_bs_store* bs, Ring* ring) {
  if (bs->ring != 1 || bs->ring_store == nullptr) return SGB_ERR_ARG;
  if (bs->iz0 < 0 || bs->ix0 < 0 || bs->iz1 > g->nz || bs->ix1 > g->nx || bs->iz0 >= bs->iz1 || bs->ix0 >= bs->ix1)
    return SGB_ERR_SHAPE;
  *ring = make_ring(*g, bs->iz0, bs->iz1, bs->ix0, bs->ix1, 1);
  if (ring->size != bs->ring_size) return SGB_ERR_SHAPE;
  if (bs->ckpt_every > 0 && bs->ckpt_store == nullptr) return SGB_ERR_ARG;
  return SGB_OK;
}

}  // namespace

extern "C" {

int sgb_elastic_coefficients(const sgb_grid* grid, const float* vp, const float* vs, const float* rho,
                             const float* damp, float* coef_out, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (vp == nullptr || vs == nullptr || rho == nullptr || damp == nullptr || coef_out == nullptr) return SGB_ERR_ARG;
  if (!aligned16(coef_out)) return SGB_ERR_ALIGN;
  SGB_CUDA_CHECK(launch_elastic_coef(*grid, vp, vs, rho, damp, coef_out, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_elastic_step(const sgb_grid* grid, const sgb_elastic_model* model, const float* const in[5],
                     float* const out[5], sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_emodel(model)) return e;
  if (int e = check_fields(in, 5)) return e;
  if (int e = check_fields(out, 5)) return e;
  ElFwdArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_geometry(a, grid);
  for (int f = 0; f < 5; ++f) {
    a.in[f] = in[f];
    a.out[f] = out[f];
  }
  a.c = coef_planes(grid, model);
  a.status = status_ptr();
  SGB_CUDA_CHECK(launch_elastic_fwd(a, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_elastic_step_vjp(const sgb_grid* grid, const sgb_elastic_model* model, const float* const vin[2],
                         const float* const sout[3], const float* const gout[5], float* const gin[5],
                         float* const grad_shot[3], sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_emodel(model)) return e;
  if (int e = check_fields(vin, 2)) return e;
  if (int e = check_fields(sout, 3)) return e;
  if (int e = check_fields(gout, 5)) return e;
  if (int e = check_fields(gin, 5)) return e;
  if (int e = check_fields(grad_shot, 3)) return e;
  ElBwdArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_geometry(a, grid);
  // mode 1 reads the output stresses through s_in[2..4]
  a.s_in[2] = sout[0];
  a.s_in[3] = sout[1];
  a.s_in[4] = sout[2];
  a.s_in[0] = a.s_in[1] = sout[0];  // unused in mode 1
  a.v_in[0] = vin[0];
  a.v_in[1] = vin[1];
  for (int f = 0; f < 5; ++f) {
    a.a_in[f] = gout[f];
    a.a_out[f] = gin[f];
  }
  for (int k = 0; k < 3; ++k) a.grad[k] = grad_shot[k];
  a.c = coef_planes(grid, model);
  a.status = status_ptr();
  SGB_CUDA_CHECK(launch_elastic_bwd(a, 1, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_elastic_forward(const sgb_grid* grid, const sgb_elastic_model* model, const sgb_acquisition* acq,
                        const sgb_elastic_io* io, float* const buf[10], float* illum, const sgb_bs_store* bs,
                        int32_t* cur_out, sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_emodel(model)) return e;
  if (int e = check_acq(grid, acq)) return e;
  if (int e = check_io(io, acq)) return e;
  if (int e = check_fields(buf, 10)) return e;
  if (cur_out == nullptr) return SGB_ERR_ARG;
  if ((acq->nsrc > 0 && acq->src_zr == nullptr) || (acq->records != nullptr && acq->rec_zr == nullptr))
    return SGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  ElFwdArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_geometry(a, grid);
  a.c = coef_planes(grid, model);
  fill_points(a.p, acq, io);
  a.illum = illum;
  a.illum_field = io->illum_field;
  a.status = status_ptr();
  const long long field = (long long)grid->nz * grid->pitch * grid->nshots;
  if (bs != nullptr) {
    if (int e = check_bs(grid, bs, &a.ring)) return e;
  }
  int cur = 0;
  for (int t = 0; t < acq->nt; ++t) {
    for (int f = 0; f < 5; ++f) {
      a.in[f] = buf[5 * cur + f];
      a.out[f] = buf[5 * (1 - cur) + f];
    }
    a.p.t = t;
    a.records = acq->records ? acq->records + (long long)t * acq->nrec * acq->nch : nullptr;
    a.ring_out = bs ? bs->ring_store + (long long)t * 5 * grid->nshots * a.ring.size : nullptr;
    SGB_CUDA_CHECK(launch_elastic_fwd(a, s));
    cur = 1 - cur;
    if (bs != nullptr && bs->ckpt_every > 0 && (t + 1) % bs->ckpt_every == 0) {
      float* slot = bs->ckpt_store + (long long)((t + 1) / bs->ckpt_every - 1) * 5 * field;
      for (int f = 0; f < 5; ++f)
        SGB_CUDA_CHECK(cudaMemcpyAsync(slot + f * field, buf[5 * cur + f], field * sizeof(float),
                                       cudaMemcpyDeviceToDevice, s));
    }
  }
  *cur_out = cur;
  return SGB_OK;
}

int sgb_elastic_gradient(const sgb_grid* grid, const sgb_elastic_model* model, const float* const grad_shot[3],
                         const float* vp, const float* vs, const float* rho, const sgb_bs_store* bs, int32_t box,
                         float* const grad_out[3], sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_emodel(model)) return e;
  if (int e = check_fields(grad_shot, 3)) return e;
  if (vp == nullptr || vs == nullptr || rho == nullptr || grad_out == nullptr) return SGB_ERR_ARG;
  if (box && bs == nullptr) return SGB_ERR_ARG;
  const int iz0 = box ? bs->iz0 : 0, iz1 = box ? bs->iz1 : grid->nz;
  const int ix0 = box ? bs->ix0 : 0, ix1 = box ? bs->ix1 : grid->nx;
  SGB_CUDA_CHECK(launch_elastic_grad(*grid, model->coef, grad_shot, vp, vs, rho, box ? 1 : 0, iz0, iz1, ix0, ix1,
                                     grad_out, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_elastic_backward(const sgb_grid* grid, const sgb_elastic_model* model, const sgb_acquisition* acq,
                         const sgb_elastic_io* io, const sgb_bs_store* bs, float* const sbuf[10], int32_t scur,
                         float* const abuf[10], float* const grad_shot[3], const float* vp, const float* vs,
                         const float* rho, float* const grad_out[3], sgb_stream_t stream) {
  if (int e = check_grid(grid)) return e;
  if (int e = check_emodel(model)) return e;
  if (int e = check_acq(grid, acq)) return e;
  if (int e = check_io(io, acq)) return e;
  if (int e = check_fields(sbuf, 10)) return e;
  if (int e = check_fields(abuf, 10)) return e;
  if (int e = check_fields(grad_shot, 3)) return e;
  if (bs == nullptr || scur < 0 || scur > 1) return SGB_ERR_ARG;
  if ((acq->nsrc > 0 && acq->src_zr == nullptr) || (acq->records != nullptr && acq->rec_zr == nullptr))
    return SGB_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  ElBwdArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_geometry(a, grid);
  if (int e = check_bs(grid, bs, &a.ring)) return e;
  a.c = coef_planes(grid, model);
  fill_points(a.p, acq, io);
  a.status = status_ptr();
  const long long field = (long long)grid->nz * grid->pitch * grid->nshots;
  for (int f = 0; f < 10; ++f) SGB_CUDA_CHECK(cudaMemsetAsync(abuf[f], 0, field * sizeof(float), s));
  // the reverse loop adds every shot's gradient terms into plane 0 of each field
  for (int k = 0; k < 3; ++k) {
    SGB_CUDA_CHECK(cudaMemsetAsync(grad_shot[k], 0, (long long)grid->nz * grid->pitch * sizeof(float), s));
    a.grad[k] = grad_shot[k];
  }
  const int nt = acq->nt;
  const int K = bs->ckpt_every;
  const int nslots = K > 0 ? nt / K : 0;
  int sc = scur, ac = 0;
  for (int i = nt - 1; i >= 0; --i) {
    for (int f = 0; f < 5; ++f) {
      a.s_in[f] = sbuf[5 * sc + f];
      a.s_out[f] = sbuf[5 * (1 - sc) + f];
      a.a_in[f] = abuf[5 * ac + f];
      a.a_out[f] = abuf[5 * (1 - ac) + f];
    }
    a.p.t = i;
    a.resid = acq->records ? acq->records + (long long)i * acq->nrec * acq->nch : nullptr;
    a.ring_in = i >= 1 ? bs->ring_store + (long long)(i - 1) * 5 * grid->nshots * a.ring.size : nullptr;
    SGB_CUDA_CHECK(launch_elastic_bwd(a, 0, s));
    sc = 1 - sc;
    ac = 1 - ac;
    if (K > 0 && i % K == 0 && i / K >= 1 && i / K <= nslots) {
      const float* slot = bs->ckpt_store + (long long)(i / K - 1) * 5 * field;
      for (int f = 0; f < 5; ++f)
        SGB_CUDA_CHECK(cudaMemcpyAsync(sbuf[5 * sc + f], slot + f * field, field * sizeof(float),
                                       cudaMemcpyDeviceToDevice, s));
    }
  }
  if (grad_out != nullptr && vp != nullptr && vs != nullptr && rho != nullptr) {
    const float* gs[3] = {grad_shot[0], grad_shot[1], grad_shot[2]};
    sgb_grid one = *grid;
    one.nshots = 1;
    SGB_CUDA_CHECK(launch_elastic_grad(one, model->coef, gs, vp, vs, rho, 1, bs->iz0, bs->iz1, bs->ix0, bs->ix1,
                                       grad_out, s));
  }
  return SGB_OK;
}

}  // extern "C"
