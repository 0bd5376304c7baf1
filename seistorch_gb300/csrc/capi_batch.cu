// extern "C" entry points of the uneven-batch forward (several grids, one
// persistent launch per step) and its CUDA-graph plan.
#include <cstring>
#include <new>
#include <vector>

#include "sgb_common.cuh"
#include "acoustic_args.cuh"
#include "capi_util.cuh"
#include "tma.cuh"

namespace sgb {
FdWeights fd_weights(int order);
int field_map(CUtensorMap* m, const float* p, int nz, int nx, int pitch, int nshots, int boxw, int rb,
              int bs = 1);
int fwd_tile_rows();
int stencil_box_width(int R);
cudaError_t launch_acoustic_fwd_batch(int R, const AcFwdBatch<MAX_BATCH_GROUPS>& b, cudaStream_t s);
cudaError_t prepare_acoustic_fwd_batch(int R);
}  // namespace sgb

using namespace sgb;

struct sgb_plan_st {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

struct GroupMaps {
  CUtensorMap stencil[3];  // haloed rows of each rotating buffer
  CUtensorMap point[3];    // point boxes of each rotating buffer
};

int check_group(const sgb_batch_group& g, int order) {
  if (int e = check_grid(&g.grid)) return e;
  if (int e = check_acq(&g.grid, &g.acq)) return e;
  const sgb_acoustic_model& m = g.model;
  if (m.coef == nullptr) return SGB_ERR_ARG;
  if (m.boundary != 0) return SGB_ERR_UNSUPPORTED;  // the batch covers the PML equation
  if (m.order != order) return SGB_ERR_UNSUPPORTED;
  if (!aligned16(m.coef)) return SGB_ERR_ALIGN;
  for (int i = 0; i < 3; ++i) {
    if (g.buf[i] == nullptr) return SGB_ERR_ARG;
    if (!aligned16(g.buf[i])) return SGB_ERR_ALIGN;
  }
  if (g.acq.records != nullptr && g.acq.nch != 1) return SGB_ERR_UNSUPPORTED;
  if ((g.acq.nsrc > 0 && g.acq.src_zr == nullptr) || (g.acq.records != nullptr && g.acq.rec_zr == nullptr))
    return SGB_ERR_ARG;
  return SGB_OK;
}

AcStreamArgs group_args(const sgb_batch_group& G, int tzr) {
  AcStreamArgs a;
  std::memset(&a, 0, sizeof(a));
  const sgb_grid& g = G.grid;
  a.nz = g.nz;
  a.nx = g.nx;
  a.pitch = g.pitch;
  a.nshots = g.nshots;
  a.ntx = (g.nx + TX - 1) / TX;
  a.zc = tzr;
  a.nzc = (g.nz + tzr - 1) / tzr;
  a.nseg = a.nzc;
  a.tpu = 1;
  const long long plane = (long long)g.nz * g.pitch;
  a.g = G.model.coef;
  a.k = G.model.coef + plane;
  a.src_zr = G.acq.src_zr;
  a.rec_zr = G.acq.rec_zr;
  a.sstride = plane;
  a.w = fd_weights(G.model.order);
  a.src_ptr = G.acq.nsrc > 0 ? G.acq.src_ptr : nullptr;
  a.src_z = G.acq.src_z;
  a.src_x = G.acq.src_x;
  a.src_wrow = G.acq.src_wrow;
  a.wavelet = G.acq.wavelet;
  a.nt = G.acq.nt;
  a.rec_row_ptr = G.acq.rec_row_ptr;
  a.rec_x = G.acq.rec_x;
  a.rec_col = G.acq.rec_col;
  a.nrec = G.acq.nrec;
  a.nch = G.acq.nch;
  a.illum = G.illum;
  a.status = status_ptr();
  return a;
}

// Issues the whole uneven loop on stream s (zeroing first when `zero`).
int run_batch(const sgb_batch_group* groups, int ng, int32_t* cur_out, int32_t* prev_out, cudaStream_t s,
              bool zero) {
  if (groups == nullptr || ng < 1 || ng > MAX_BATCH_GROUPS) return SGB_ERR_ARG;
  const int order = groups[0].model.order;
  if (order != 2 && order != 4 && order != 6 && order != 8) return SGB_ERR_UNSUPPORTED;
  for (int g = 0; g < ng; ++g)
    if (int e = check_group(groups[g], order)) return e;
  const int R = order / 2;
  const int tzr = fwd_tile_rows();
  const int bw = stencil_box_width(R);
  std::vector<GroupMaps> maps(ng);
  std::vector<AcStreamArgs> args(ng);
  int nt_max = 0;
  for (int g = 0; g < ng; ++g) {
    const sgb_batch_group& G = groups[g];
    for (int i = 0; i < 3; ++i)
      if (field_map(&maps[g].stencil[i], G.buf[i], G.grid.nz, G.grid.nx, G.grid.pitch, G.grid.nshots, bw,
                    tzr + 2 * R) ||
          field_map(&maps[g].point[i], G.buf[i], G.grid.nz, G.grid.nx, G.grid.pitch, G.grid.nshots, TX, tzr))
        return SGB_ERR_CUDA;
    args[g] = group_args(G, tzr);
    nt_max = G.acq.nt > nt_max ? G.acq.nt : nt_max;
  }
  if (zero) {
    for (int g = 0; g < ng; ++g) {
      const sgb_grid& gr = groups[g].grid;
      const size_t field = (size_t)gr.nshots * gr.nz * gr.pitch * sizeof(float);
      for (int i = 0; i < 3; ++i) SGB_CUDA_CHECK(cudaMemsetAsync(groups[g].buf[i], 0, field, s));
      if (groups[g].illum != nullptr)
        SGB_CUDA_CHECK(cudaMemsetAsync(groups[g].illum, 0, (size_t)gr.nz * gr.pitch * sizeof(float), s));
    }
  }
  AcFwdBatch<MAX_BATCH_GROUPS> b;
  std::memset(&b, 0, sizeof(b));
  int cur = 0, prev = 1, nxt = 2;
  for (int t = 0; t < nt_max; ++t) {
    int k = 0;
    b.tile0[0] = 0;
    for (int g = 0; g < ng; ++g) {
      const sgb_batch_group& G = groups[g];
      if (t >= G.acq.nt) continue;
      b.tm_u[k] = maps[g].stencil[cur];
      b.tm_um[k] = maps[g].point[prev];
      AcStreamArgs a = args[g];
      a.um = G.buf[prev];
      a.un = G.buf[nxt];
      a.t = t;
      a.records = G.acq.records ? G.acq.records + (long long)t * G.acq.nrec * G.acq.nch : nullptr;
      b.g[k] = a;
      b.tile0[k + 1] = b.tile0[k] + a.nshots * a.ntx * a.nzc;
      ++k;
    }
    b.ngroups = k;
    SGB_CUDA_CHECK(launch_acoustic_fwd_batch(R, b, s));
    prev = cur;
    cur = nxt;
    nxt = 3 - prev - cur;
    for (int g = 0; g < ng; ++g)
      if (t + 1 == groups[g].acq.nt && cur_out != nullptr && prev_out != nullptr) {
        cur_out[g] = cur;
        prev_out[g] = prev;
      }
  }
  return SGB_OK;
}

}  // namespace

extern "C" {

int sgb_acoustic_batch_forward(const sgb_batch_group* groups, int32_t ngroups, int32_t* cur_out, int32_t* prev_out,
                               sgb_stream_t stream) {
  if (groups == nullptr || ngroups < 1) return SGB_ERR_ARG;
  SGB_CUDA_CHECK(prepare_acoustic_fwd_batch(groups[0].model.order / 2));
  return run_batch(groups, ngroups, cur_out, prev_out, (cudaStream_t)stream, true);
}

int sgb_acoustic_batch_plan(const sgb_batch_group* groups, int32_t ngroups, int32_t* cur_out, int32_t* prev_out,
                            sgb_plan* plan_out) {
  if (plan_out == nullptr || groups == nullptr || ngroups < 1) return SGB_ERR_ARG;
  *plan_out = nullptr;
  // kernel attributes are set outside the capture
  SGB_CUDA_CHECK(prepare_acoustic_fwd_batch(groups[0].model.order / 2));
  cudaStream_t cs = nullptr;
  SGB_CUDA_CHECK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  sgb_plan plan = new (std::nothrow) sgb_plan_st;
  if (plan == nullptr) {
    cudaStreamDestroy(cs);
    return SGB_ERR_ARG;
  }
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  int st = SGB_OK;
  if (e == cudaSuccess) {
    st = run_batch(groups, ngroups, cur_out, prev_out, cs, true);
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    if (st == SGB_OK && e2 != cudaSuccess) st = set_cuda_error(e2);
    plan->graph = graph;
    if (st == SGB_OK) {
      const cudaError_t e3 = cudaGraphInstantiate(&plan->exec, graph, 0);
      if (e3 != cudaSuccess) st = set_cuda_error(e3);
    }
  } else {
    st = set_cuda_error(e);
  }
  cudaStreamDestroy(cs);
  if (st != SGB_OK) {
    sgb_plan_destroy(plan);
    return st;
  }
  *plan_out = plan;
  return SGB_OK;
}

int sgb_plan_launch(sgb_plan plan, sgb_stream_t stream) {
  if (plan == nullptr || plan->exec == nullptr) return SGB_ERR_ARG;
  SGB_CUDA_CHECK(cudaGraphLaunch(plan->exec, (cudaStream_t)stream));
  return SGB_OK;
}

int sgb_plan_destroy(sgb_plan plan) {
  if (plan == nullptr) return SGB_OK;
  if (plan->exec != nullptr) cudaGraphExecDestroy(plan->exec);
  if (plan->graph != nullptr) cudaGraphDestroy(plan->graph);
  delete plan;
  return SGB_OK;
}

}  // extern "C"
