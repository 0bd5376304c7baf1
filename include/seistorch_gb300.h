/*
 * seistorch_gb300 -- C ABI of the GB300 (sm_103a) wave-propagation hot path.
 *
 * Drop-in native layer for seistorch's 2D time stepping (the equation modules
 * seistorch/equations2d/{acoustic,acoustic_habc,elastic}.py and the loop in
 * seistorch/rnn.py + seistorch/cell.py).  Plain pointers, sizes and a
 * cudaStream_t only; no torch types.  All pointers are device pointers unless
 * a field says otherwise.  Every entry point returns an sgb_status.
 *
 * Layout: wavefields are float32 [nshots][nz][pitch] (x fastest), models and
 * coefficient planes float32 [nz][pitch]; pitch is a multiple of 4 floats
 * and >= nx; columns nx..pitch-1 are never read as data (zero padding is
 * implied, as conv2d(padding=order/2) in acoustic.py:71).
 */
#ifndef SEISTORCH_GB300_H
#define SEISTORCH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *sgb_stream_t; /* == cudaStream_t */

typedef enum {
  SGB_OK = 0,
  SGB_ERR_ARG = 1,         /* null pointer / bad enum / bad size              */
  SGB_ERR_SHAPE = 2,       /* inconsistent nz/nx/pitch/nshots                 */
  SGB_ERR_ALIGN = 3,       /* pointer not 16-byte aligned / pitch % 4 != 0    */
  SGB_ERR_CUDA = 4,        /* a CUDA runtime call failed (see sgb_last_cuda_error) */
  SGB_ERR_UNSUPPORTED = 5, /* order / option outside what the kernels cover   */
  SGB_ERR_NONFINITE = 6,   /* NaN/Inf found in records (rnn.py:215 -> type.py:41-46) */
  SGB_ERR_CAPACITY = 7,    /* too many sources inside one tile                */
  SGB_ERR_SCRATCH = 8,     /* problem larger than the fixed scratch of an
                              allocation-free entry point                    */
  SGB_ERR_CFL = 9          /* vmax * dt / h above the scheme's stability limit */
} sgb_status;

/* Grid shared by every equation. dt, h in seconds / metres. */
typedef struct {
  int32_t nz, nx;    /* padded grid (interior + boundary layers)          */
  int32_t pitch;     /* row stride in floats                              */
  int32_t nshots;    /* batch of shots (wavefield leading dimension)      */
  float dt, h;
} sgb_grid;

/* Acquisition for one time loop (rnn.py:158-212, source.py:47-57,
 * probe.py:42-44).  The optional per-shot row ranges let the kernels skip
 * the source / receiver lookups for tiles away from them.
 * Sources: CSR by shot; each point receives
 * wavelet[wrow * nt + t] at step t (the smask*X add; the caller removes
 * duplicate points within a shot, as the 0/1 mask does).  Receivers: CSR by
 * (shot, row) -- rec_row_ptr[b * nz + z] .. rec_row_ptr[b * nz + z + 1] --
 * each with its column x and its output column in records[t][col][ch]. */
typedef struct {
  const int32_t *src_ptr;     /* [nshots + 1]                         */
  const int32_t *src_z;       /* [nsrc]                               */
  const int32_t *src_x;       /* [nsrc]                               */
  const int32_t *src_wrow;    /* [nsrc] row of `wavelet` per source   */
  const float *wavelet;       /* [nwrows][nt]                         */
  int32_t nsrc;
  int32_t nt;
  const int32_t *rec_row_ptr; /* [nshots * nz + 1]                    */
  const int32_t *rec_x;       /* [nrec]                               */
  const int32_t *rec_col;     /* [nrec] column in the record matrix   */
  int32_t nrec;               /* record matrix width                  */
  int32_t nch;                /* channels per record (receiver types) */
  float *records;             /* [nt][nrec][nch] out (may be NULL)    */
  const int32_t *src_zr;      /* [nshots][2] first source row, last+1 (nullable) */
  const int32_t *rec_zr;      /* [nshots][2] first receiver row, last+1 (nullable) */
} sgb_acquisition;

/* 2nd-order-in-time acoustic model (acoustic.py:73-86, acoustic_habc.py:206-221).
 * coef = [g plane | k plane] from sgb_acoustic_coefficients:
 *   u+ = g (u - u-) + u- + k * L(u),  g = 2/(1 + d dt),
 *   k = vp^2 dt^2 / (h^2 (1 + d dt)),  L = cross stencil of `order`
 * (PML: d = damping; HABC: d = 0 in the update, `damp` is the blend
 * weight of habc.py:42-81). */
typedef struct {
  int32_t order;        /* 2, 4, 6 or 8                                       */
  int32_t boundary;     /* 0 = PML, 1 = HABC                                   */
  int32_t habc_width;   /* 50 (acoustic_habc.py:79, habc.py); HABC with 0: no
                           blend -- the plain undamped update of the reverse
                           steps (acoustic_habc.py:223-268)                   */
  int32_t multiple;     /* free surface at the top (no top absorbing layer)    */
  const float *coef;    /* [2][nz][pitch]                                      */
  const float *vp;      /* [nz][pitch] (HABC one-way coefficients)            */
  const float *damp;    /* [nz][pitch] PML d or HABC blend weight             */
} sgb_acoustic_model;

/* Boundary-saving store for the adjoint (checkpoint_new.py:109-217 saves
 * 1-cell strips; here `ring` cells on every side of the undamped interior
 * box [iz0,iz1) x [ix0,ix1), clipped to the grid) plus full checkpoints of
 * (U_n, U_{n-1}) every ckpt_every steps. */
typedef struct {
  int32_t iz0, iz1, ix0, ix1;
  int32_t ring;
  int32_t ring_size;        /* floats per shot per step (sgb_ring_size)     */
  float *ring_store;        /* [nt][nshots][ring_size]                      */
  int32_t ckpt_every;       /* 0: none                                      */
  float *ckpt_store;        /* [nt / ckpt_every][2][nshots][nz][pitch]      */
  float *habc_planes;       /* HABC adjoints: [5][nz][pitch] scratch for each
                               cell's interior share and its four sides'
                               shares (filled once per backward call), or
                               NULL (then evaluated on the fly each step)  */
} sgb_bs_store;

/* Library identification and diagnostics. */
const char *sgb_version(void);
const char *sgb_status_string(int status);
int sgb_last_cuda_error(void);

/* Reads (and with reset != 0 clears) the device status word that kernels set
 * (bit 1: too many sources in one tile; bit 2: an mbarrier wait ran out of
 * polls and the kernel stopped early).  Synchronous. */
int sgb_device_status(int *out, int reset);

/* Stability check of the explicit time stepping (host-only, no GPU work).
 * The reference has no such check (a too-large dt shows up as NaN records,
 * type.py:41-46); here the Python layer calls it before every loop.
 * scheme 0: 2nd-order-in-time acoustic family with the cross stencil of
 * `order` (2/4/6/8; acoustic.py:60-86) -- vmax * dt / h <= 2 / sqrt(max
 * eigenvalue of -h^2 L) (0.707, 0.612, 0.575, 0.555 for orders 2/4/6/8);
 * scheme 1: the elastic velocity-stress staggered grid (elastic.py:7-37,
 * order 2) -- vmax * dt / h <= 1/sqrt(2).  Writes the Courant number and
 * the limit (either pointer may be NULL); returns SGB_ERR_CFL above it. */
int sgb_cfl_check(int32_t scheme, int32_t order, float vmax, float dt, float h, float *courant_out,
                  float *limit_out);

/* Diagnostic of the bounded waits (no counterpart in the reference): one
 * block waits on an mbarrier for at most `polls` polls (1 .. 2^21).  With
 * arrive = 0 nothing completes the barrier, the wait runs out, sets bit 2 of
 * the device status word and the kernel returns; with arrive != 0 the wait
 * succeeds and sets nothing.  No copy is ever in flight. */
int sgb_debug_wait_probe(uint32_t polls, int32_t arrive, sgb_stream_t stream);

/* Select the tile-pipeline variants used by later calls (host-only,
 * process-wide): fwd_cfg in [0, 6) and bwd_cfg in [0, 6) index the compiled
 * (rows per tile, warps per CTA, pipeline stages, which point operands
 * travel through the TMA stage) variants of the PML forward and adjoint; habc_cfg in [0, 6) those of the second-order HABC
 * forward (plain, Born, viscoacoustic), 0 = the default.  The autotuner
 * (seistorch_gb300.tuning) times the PML variants per grid. */
int sgb_set_stream_config(int32_t fwd_cfg, int32_t bwd_cfg, int32_t habc_cfg);

/* Floats per shot per step of the boundary ring (host-only helper). */
int sgb_ring_size(const sgb_grid *grid, int32_t iz0, int32_t iz1, int32_t ix0, int32_t ix1,
                  int32_t ring, int32_t *size_out);

/* Coefficient planes for sgb_acoustic_model.coef.  Replaces the per-step
 * (dt^-2 + b/dt)^-1 and c.pow(2) work of acoustic.py:81-84. */
int sgb_acoustic_coefficients(const sgb_grid *grid, const float *vp, const float *damp,
                              int32_t boundary, float *coef_out, sgb_stream_t stream);

/* One time step: unext = step(u, um).  Replaces acoustic._time_step
 * (acoustic.py:73-86) and acoustic_habc._time_step (acoustic_habc.py:206-221);
 * unext must not alias u or um. */
int sgb_acoustic_step(const sgb_grid *grid, const sgb_acoustic_model *model, const float *u,
                      const float *um, float *unext, sgb_stream_t stream);

/* Vector-Jacobian product of one PML step (autograd of acoustic.py:73-86):
 * given gy = dJ/dy and gh1 = dJ/d(second output h1), writes
 * gu = dJ/du (h1), gum = dJ/dum (h2) and accumulates gvp_acc += sum over
 * shots of gy * L(u) (caller multiplies by 2k/vp).  gh1 may be NULL. */
int sgb_acoustic_step_vjp(const sgb_grid *grid, const sgb_acoustic_model *model, const float *u,
                          const float *gy, const float *gh1, float *gu, float *gum,
                          float *gvp_acc, sgb_stream_t stream);

/* Inputs and outputs of sgb_habc_step_vjp.  Fields [nshots][nz][pitch],
 * planes [nz][pitch]; outputs are overwritten. */
typedef struct {
  const float *u;      /* U_n (h1 / p1)                                           */
  const float *um;     /* U_{n-1} (h2 / p2)                                       */
  const float *gy;     /* dJ/dy of the step's output                              */
  float *gu;           /* out dJ/dU_n                                             */
  float *gum;          /* out dJ/dU_{n-1}                                         */
  float *gparam;       /* out sum over shots of wi * gy * dI/dtheta, I the interior
                          update: 1 plane (L(U)) for the plain equation and Born,
                          2 for VTI (Lx(U), Lz(U)), 5 for variable density
                          (D(U), C dx+U, -C dx-U, C dz+U, -C dz-U)                */
  float *gvp_oneway;   /* out sum over shots of gy * d(one-way blend)/dvp, or NULL
                          (unused when model->habc_width == 0)                    */
  const float *kz;     /* VTI: the z coefficient plane (coef = [g][kx][kz]), else NULL */
  const float *rho_c;  /* variable density: planes C, bx+, bx-, bz+, bz-, else NULL  */
  const float *born_m; /* Born, scattered field: reflectivity m, else NULL        */
  const float *born_u; /* Born: the background field U_n of the m k L(U) source   */
  float *born_gu;      /* Born: out dJ/d(background U_n) through the source       */
  float *born_gm;      /* Born: out dJ/dm (plane)                                 */
  float *wi_out;       /* out: each cell's interior share wi = 1 - b sum of its
                          sides' shares (plane), or NULL                          */
} sgb_habc_vjp_io;

/* Vector-Jacobian product of one step of the HABC family (autograd of
 * acoustic_habc._time_step, acoustic_habc.py:206-221; vti_habc2._time_step,
 * vti_habc2.py:25-60; acoustic_rho_habc._time_step, acoustic_rho_habc.py:31-58;
 * one field of acoustic_lsrtm_habc._time_step, acoustic_lsrtm_habc.py:11-30):
 * the transposed interior update weighted by each cell's interior share, the
 * transposed one-way blends of the four strips (mask precedence, corner
 * halves, the depth-49 roll wrap), over the whole grid.  model->boundary must
 * be 1; habc_width 0 gives the VJP of the unblended reverse step
 * (acoustic_habc.py:223-268).  The caller maps gparam through the
 * coefficient map (k = vp^2 dt^2 / h^2: dJ/dvp += gparam * 2k / vp) and adds
 * gvp_oneway to dJ/dvp. */
int sgb_habc_step_vjp(const sgb_grid *grid, const sgb_acoustic_model *model, const sgb_habc_vjp_io *io,
                      sgb_stream_t stream);

/* Whole time loop (rnn.py:178-205) in one call: nt steps of the model with
 * source injection and receiver sampling fused into the step kernel.
 * buf[0..2] are three [nshots][nz][pitch] buffers; on entry buf[0] = U_0 and
 * buf[1] = U_{-1} (zeros for a cold start).  On return *cur_out / *prev_out
 * index the buffers holding U_nt and U_{nt-1}.  illum (nullable, [nz][pitch])
 * accumulates sum_b u^2 of the source field (rnn.py:204-205).  bs (nullable)
 * saves the boundary ring every step and checkpoints every ckpt_every. */
int sgb_acoustic_forward(const sgb_grid *grid, const sgb_acoustic_model *model,
                         const sgb_acquisition *acq, float *const buf[3], float *illum,
                         const sgb_bs_store *bs, int32_t *cur_out, int32_t *prev_out,
                         sgb_stream_t stream);

/* Adjoint of sgb_acoustic_forward (PML or HABC): boundary-saving
 * reconstruction of the forward wavefield in the interior box + adjoint time
 * stepping + vp gradient, in one fused kernel per step (PML: TMA tile
 * pipeline; HABC: a tiled kernel that also applies the transposed
 * one-way boundary blend, acoustic_habc.py:79-204; model->vp and
 * model->damp = the HABC weights are required).  Replaces the autograd path
 * of checkpoint_new.py:146-217 with an exact discrete adjoint.
 *   ubuf[0..2]: [nshots][nz][pitch]; on entry ubuf[ucur] = U_nt and
 *               ubuf[uprev] = U_{nt-1} (as left by sgb_acoustic_forward);
 *   lbuf[0..2]: [nshots][nz][pitch] adjoint scratch (zeroed here);
 *   acq->records: dJ/d(records) [nt][nrec][nch] (the adjoint source);
 *   grad_shot: [nshots][nz][pitch] scratch: the adjoint adds every shot's
 *              gradient term into its first [nz][pitch] plane (zeroed here)
 *              with reduction atomics, so the order of the sum over shots
 *              is not fixed;
 *   grad_vp: [nz][pitch] out, dJ/dvp inside the interior box, 0 outside. */
int sgb_acoustic_backward(const sgb_grid *grid, const sgb_acoustic_model *model,
                          const sgb_acquisition *acq, const sgb_bs_store *bs,
                          float *const ubuf[3], int32_t ucur, int32_t uprev,
                          float *const lbuf[3], float *grad_shot, float *grad_vp,
                          sgb_stream_t stream);

/* Allocation-free adjoint.  No counterpart in the reference: an addition for
 * callers that cannot allocate device memory themselves (a host application
 * or plugin framework that owns all device memory and forbids cudaMalloc /
 * cudaFree on its threads, or a loop that must not allocate while it runs).
 * Same contract as sgb_acoustic_backward, without the lbuf / grad_shot
 * scratch arguments: the scratch lives in a fixed 32 MiB device array inside
 * this library (held by every GPU that loads it until the process exits), so
 * 4 * nshots * nz * pitch must not exceed 8,388,608 floats; larger problems
 * return SGB_ERR_SCRATCH before any work.  The first call on a device looks
 * up the array's address there (cudaGetSymbolAddress with that device
 * current); make that first call before any stream capture.  The address
 * is cached per device for the life of the process: after cudaDeviceReset
 * on a device, do not call this entry point on that device again.  All calls share
 * the one array, which keeps the last call's contents (the adjoint clears what
 * must start at zero), so calls that overlap on the GPU -- on different
 * streams or threads -- race and must be serialised by the caller.  No
 * cudaMalloc, cudaFree or allocating library routine is called. */
int sgb_acoustic_backward_noalloc(const sgb_grid *grid, const sgb_acoustic_model *model,
                                  const sgb_acquisition *acq, const sgb_bs_store *bs,
                                  float *const ubuf[3], int32_t ucur, int32_t uprev, float *grad_vp,
                                  sgb_stream_t stream);

/* ---------------------------------------------------- viscoacoustic --- */

/* The viscoacoustic equation with the HABC (vacoustic_habc.py:74-115):
 *   y = HABC(2U - U- + kv L(U) + a_neg K(U - U-)) + sources,
 * K(x) = real(ifft2(|k| fft2(x))) over the padded grid, |k| =
 * sqrt(fz^2 + fx^2) with fz / fx = fftfreq(nz / nx, h), kv =
 * vp^2 dt^2 (1 - (1 - sqrt(Q^2 + 1)) / Q^2) / h^2 and a_neg = -dt t vp / 2
 * with the reference's t(Q, omega) (the caller computes both planes;
 * model->coef = [g = 2][kv]).  Scratch (caller-allocated):
 * sgb_vacoustic_work_size floats of complex work and twiddles. */
int sgb_vacoustic_work_size(const sgb_grid *grid, int64_t *work_floats, int64_t *tw_floats);

/* out[b] = post * K(pre * (u1[b] - u2[b])) for every shot; pre, u2, post may
 * be NULL (1, 0, 1).  Two shots share one complex transform (K is real and
 * even); mixed-radix transforms, nz, nx <= 8192.  out must not alias u1/u2. */
int sgb_vacoustic_kterm(const sgb_grid *grid, const float *pre, const float *u1, const float *u2,
                        const float *post, float *out, float *work, float *tw, sgb_stream_t stream);

/* One step of vacoustic_habc._time_step (no sources): unext = step(u, um);
 * extra receives a_neg K(u - um). */
int sgb_vacoustic_step(const sgb_grid *grid, const sgb_acoustic_model *model, const float *a_neg, const float *u,
                       const float *um, float *unext, float *extra, float *work, float *tw, sgb_stream_t stream);

/* Whole forward loop of vacoustic_habc (records; as sgb_acoustic_forward
 * with the damping term; no boundary store).  extra: one field of scratch. */
int sgb_vacoustic_forward(const sgb_grid *grid, const sgb_acoustic_model *model, const float *a_neg,
                          const sgb_acquisition *acq, float *const buf[3], float *extra, float *work, float *tw,
                          int32_t *cur_out, int32_t *prev_out, sgb_stream_t stream);

/* ---------------------------------------------------------------- VTI --- */

/* The loop of vti_habc2._time_step (seistorch/equations2d/vti_habc2.py:26-56),
 * second order, HABC: U+ = HABC(2U - U- + kx Lx(U) + kz Lz(U)) + sources,
 * Lx / Lz the 1-D second differences along x / z (convkernel.py kernelx /
 * kernely).  model->coef holds THREE planes [g][kx][kz] (g = 2 everywhere,
 * kx = vp^2 dt^2 (1 + 2 eps + sk) / h^2, kz = vp^2 dt^2 (1 + sk) / h^2 with
 * the reference's per-cell sk of eps, delta and the cell's FFT frequencies;
 * the caller computes them); model->order must be 2 and model->boundary 1.
 * Other arguments as sgb_acoustic_forward (no illumination). */
int sgb_vti_forward(const sgb_grid *grid, const sgb_acoustic_model *model, const sgb_acquisition *acq,
                    float *const buf[3], const sgb_bs_store *bs, int32_t *cur_out, int32_t *prev_out,
                    sgb_stream_t stream);

/* Adjoint of sgb_vti_forward: the exact HABC adjoint with the anisotropic
 * interior update; returns dJ/dkx = sum_t La Lx(U) and dJ/dkz = sum_t La Lz(U)
 * inside the undamped box (0 outside), from which the caller forms the
 * vp / eps / delta gradients through its coefficient map.  grad_shot_x /
 * grad_shot_z: scratch [nshots][nz][pitch] each; the rest as
 * sgb_acoustic_backward. */
int sgb_vti_backward(const sgb_grid *grid, const sgb_acoustic_model *model, const sgb_acquisition *acq,
                     const sgb_bs_store *bs, float *const ubuf[3], int32_t ucur, int32_t uprev,
                     float *const lbuf[3], float *grad_shot_x, float *grad_shot_z, float *grad_x,
                     float *grad_z, sgb_stream_t stream);

/* One step (no sources or receivers): the per-step equation-module drop-in. */
int sgb_vti_step(const sgb_grid *grid, const sgb_acoustic_model *model, const float *u, const float *um,
                 float *unext, sgb_stream_t stream);

/* --------------------------------------------------- variable density --- */

/* The loop of acoustic_rho_habc._time_step
 * (seistorch/equations2d/acoustic_rho_habc.py:34-58), second order, HABC:
 * U+ = HABC(2U - U- + C (bx+ (U[x+1] - U) - bx- (U - U[x-1])
 *                        + bz+ (U[z+1] - U) - bz- (U - U[z-1]))) + sources,
 * rho_c: five planes [5][nz][pitch] = C = dt^2 rho vp^2 / h^2 and the
 * buoyancy averages bx+ = (b + b[x+1]) / 2, bx- = (b[x-1] + b) / 2,
 * bz+ = (b + b[z+1]) / 2, bz- = (b[z-1] + b) / 2 of b = 1 / rho with zeros
 * beyond the grid (the reference's zero-padded convolutions); the caller
 * computes them.  model: from sgb_acoustic_coefficients with boundary 1
 * (order 2). */
int sgb_rho_forward(const sgb_grid *grid, const sgb_acoustic_model *model, const float *rho_c,
                    const sgb_acquisition *acq, float *const buf[3], const sgb_bs_store *bs,
                    int32_t *cur_out, int32_t *prev_out, sgb_stream_t stream);

/* Adjoint of sgb_rho_forward: the exact HABC adjoint of the variable-density
 * update; grad5 receives the five planes dJ/dC, dJ/dbx+, dJ/dbx-, dJ/dbz+,
 * dJ/dbz- inside the undamped box (0 outside), for the caller's chain rule
 * to vp and rho.  grad_shot5: scratch [5][nshots][nz][pitch]. */
int sgb_rho_backward(const sgb_grid *grid, const sgb_acoustic_model *model, const float *rho_c,
                     const sgb_acquisition *acq, const sgb_bs_store *bs, float *const ubuf[3], int32_t ucur,
                     int32_t uprev, float *const lbuf[3], float *grad_shot5, float *grad5,
                     sgb_stream_t stream);

/* One step without sources or receivers (the per-step drop-in). */
int sgb_rho_step(const sgb_grid *grid, const sgb_acoustic_model *model, const float *rho_c, const float *u,
                 const float *um, float *unext, sgb_stream_t stream);

/* --------------------------------------------------- Born modelling --- */

/* Born (linearised) modelling of the acoustic HABC equation for
 * least-squares RTM: the loop of acoustic_lsrtm_habc._time_step
 * (seistorch/equations2d/acoustic_lsrtm_habc.py:11-30) with its sources on
 * the background field h1 and its receivers on the scattered field sh1
 * (examples/lsrtm/acoustic/configs/lsrtm.yml).  Per step:
 *   p+ = HABC(2p - p- + k L(p)) + sources,
 *   s+ = HABC(2s - s- + k L(s) + m k L(p)),   records sample s+;
 * model->boundary must be 1 (HABC), m is the reflectivity plane
 * [nz][pitch].  pbuf / sbuf: the background and scattered fields' three
 * rotating buffers (zeroed here; both rotate together, so cur_out /
 * prev_out name U_nt / U_{nt-1} of both); born_src: scratch
 * [nshots][nz][pitch].  bs (optional) saves the background's boundary ring
 * and checkpoints for sgb_born_backward. */
int sgb_born_forward(const sgb_grid *grid, const sgb_acoustic_model *model, const float *m,
                     const sgb_acquisition *acq, float *const pbuf[3], float *const sbuf[3],
                     float *born_src, const sgb_bs_store *bs, int32_t *cur_out, int32_t *prev_out,
                     sgb_stream_t stream);

/* One step of the same pair of fields without sources or receivers (the
 * per-step equation-module drop-in, acoustic_lsrtm_habc._time_step):
 * pnext = HABC step of (p, pm), snext = HABC step of (sc, scm) + m k L(p);
 * born_src: scratch [nshots][nz][pitch]. */
int sgb_born_step(const sgb_grid *grid, const sgb_acoustic_model *model, const float *m, const float *p,
                  const float *pm, const float *sc, const float *scm, float *pnext, float *snext,
                  float *born_src, sgb_stream_t stream);

/* dJ/dm of sgb_born_forward (the reference's autograd gradient of the
 * reflectivity, the velocity held fixed as in lsrtm.yml's invlist): the
 * exact HABC adjoint of the scattered field, driven by dJ/d(records) in
 * acq->records, against the background field reconstructed from
 * pbuf[pcur] / pbuf[pprev] and bs; grad_m = sum_t La k L(p) inside the
 * undamped box, 0 outside it.  lbuf, grad_shot: as in sgb_acoustic_backward. */
int sgb_born_backward(const sgb_grid *grid, const sgb_acoustic_model *model, const sgb_acquisition *acq,
                      const sgb_bs_store *bs, float *const pbuf[3], int32_t pcur, int32_t pprev,
                      float *const lbuf[3], float *grad_shot, float *grad_m, sgb_stream_t stream);

/* ------------------------------------------------------ uneven batch --- */

/* One grid of an uneven batch: its own shape and shots (grid), PML model,
 * acquisition (its own nt: trace lengths may differ between groups) and
 * three [nshots][nz][pitch] field buffers.  Every group must use the same
 * spatial order.  No counterpart in the reference, which runs one grid per
 * process (seistorch_dist.py:79-303); this is the batch-descriptor launch of
 * its hot path. */
typedef struct {
  sgb_grid grid;
  sgb_acoustic_model model;
  sgb_acquisition acq;
  float *buf[3];
  float *illum; /* nullable */
} sgb_batch_group;

#define SGB_MAX_BATCH_GROUPS 8

/* Time loops of up to SGB_MAX_BATCH_GROUPS grids, one persistent launch per
 * step covering the tiles of every group still running (a group stops after
 * its own nt steps).  Buffers start from zero here.  cur_out / prev_out
 * (host arrays [ngroups]) name each group's buffers holding U_nt and
 * U_{nt-1}. */
int sgb_acoustic_batch_forward(const sgb_batch_group *groups, int32_t ngroups, int32_t *cur_out,
                               int32_t *prev_out, sgb_stream_t stream);

/* The same loop recorded once as a CUDA graph (zeroing of the buffers, one
 * kernel node per step) for replay with sgb_plan_launch; replays reuse the
 * descriptors' pointers, so the buffers and tables must stay allocated and
 * in place until sgb_plan_destroy.  Records the variant current at creation
 * (sgb_set_stream_config).  cur_out / prev_out as above. */
typedef struct sgb_plan_st *sgb_plan;
int sgb_acoustic_batch_plan(const sgb_batch_group *groups, int32_t ngroups, int32_t *cur_out,
                            int32_t *prev_out, sgb_plan *plan_out);
int sgb_plan_launch(sgb_plan plan, sgb_stream_t stream);
int sgb_plan_destroy(sgb_plan plan);

/* ----------------------------------------------------------- elastic --- */

/* Field order of the elastic state, as Wavefield('elastic') lists it
 * (eqconfigure.py:45-127): vx, vz, txx, tzz, txz. */
enum { SGB_VX = 0, SGB_VZ = 1, SGB_TXX = 2, SGB_TZZ = 3, SGB_TXZ = 4, SGB_ELASTIC_FIELDS = 5 };

/* Isotropic elastic velocity-stress model (elastic.py:7-37).  coef holds
 * six planes [q | e | pa | la | ma | bv] from sgb_elastic_coefficients, with
 * c = dt d / 2, lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2:
 *   q = (1 - c) / (1 + c),  e = dt / (h (1 + c)),
 *   pa = e (lambda + 2 mu),  la = e lambda,  ma = e mu,  bv = e / rho.
 * One step (Dx-/Dz- backward, Dx+/Dz+ forward one-cell differences with the
 * first / last index zero, equations2d/utils.py:3-48):
 *   txx' = q txx + pa Dx- vx + la Dz+ vz,  tzz' = q tzz + pa Dz+ vz + la Dx- vx,
 *   txz' = q txz + ma (Dx+ vz + Dz- vx),
 *   vx'  = q vx + bv (Dx+ txx' + Dz+ txz'),  vz' = q vz + bv (Dx- txz' + Dz- tzz'). */
typedef struct {
  int32_t multiple;  /* free surface (no top absorbing layer)           */
  const float *coef; /* [6][nz][pitch]                                   */
} sgb_elastic_model;

/* Elastic source / receiver channels: src_fields is a bit mask over the
 * field order above (source_type of the config; explosive = txx | tzz);
 * rec_fields[ch] is the field that record channel ch samples (receiver_type,
 * nch <= 4); illum_field is the field whose square the illumination sums
 * (the last source type, rnn.py:204-205). */
typedef struct {
  int32_t src_fields;
  int32_t rec_fields[4];
  int32_t illum_field;
} sgb_elastic_io;

/* Coefficient planes for sgb_elastic_model.coef from vp, vs, rho and the PML
 * damping d (all [nz][pitch]); computed in double precision, zero in the
 * padding columns.  Replaces the per-step lambda / mu / (1+c)^-1 work of
 * elastic.py:11-14. */
int sgb_elastic_coefficients(const sgb_grid *grid, const float *vp, const float *vs, const float *rho,
                             const float *damp, float *coef_out, sgb_stream_t stream);

/* One step: out = step(in) (elastic._time_step, elastic.py:7-37).  in[5]
 * and out[5] are [nshots][nz][pitch] fields in the order above; out must
 * not alias in. */
int sgb_elastic_step(const sgb_grid *grid, const sgb_elastic_model *model, const float *const in[5],
                     float *const out[5], sgb_stream_t stream);

/* Vector-Jacobian product of one step (autograd of elastic._time_step):
 * given the step's input velocities vin[2] (vx, vz), its output stresses
 * sout[3] (txx', tzz', txz') and gout[5] = dJ/d(outputs), writes
 * gin[5] = dJ/d(inputs) and accumulates into grad_shot (three
 * [nshots][nz][pitch] planes: the lambda, mu and buoyancy terms before the
 * chain rule; sgb_elastic_gradient turns them into vp / vs / rho). */
int sgb_elastic_step_vjp(const sgb_grid *grid, const sgb_elastic_model *model, const float *const vin[2],
                         const float *const sout[3], const float *const gout[5], float *const gin[5],
                         float *const grad_shot[3], sgb_stream_t stream);

/* Whole elastic time loop (rnn.py:178-205): nt steps with source injection
 * and receiver sampling fused into the step kernel.  buf[0..4] and
 * buf[5..9] are two sets of five fields; set 0 holds the initial state
 * (zeros for a cold start).  On return *cur_out (0 or 1) names the set that
 * holds the final state.  bs (nullable): the ring (width 1) of all five
 * fields is saved every step ([nt][5][nshots][ring_size]) and full states
 * every ckpt_every steps ([nt / ckpt_every][5][nshots][nz][pitch]). */
int sgb_elastic_forward(const sgb_grid *grid, const sgb_elastic_model *model, const sgb_acquisition *acq,
                        const sgb_elastic_io *io, float *const buf[10], float *illum, const sgb_bs_store *bs,
                        int32_t *cur_out, sgb_stream_t stream);

/* Adjoint of sgb_elastic_forward: boundary-saving reconstruction of the
 * forward state inside the interior box, the exact discrete adjoint of the
 * step and the lambda / mu / buoyancy gradient terms, one fused kernel per
 * step.  Replaces the reconstruct-then-replay of checkpoint.py:108-230.
 *   sbuf[10], scur: the state sets as left by sgb_elastic_forward;
 *   abuf[10]: adjoint scratch (zeroed here);
 *   acq->records: dJ/d(records) [nt][nrec][nch];
 *   grad_shot[3]: [nshots][nz][pitch] accumulators (zeroed here);
 *   vp, vs, rho: the model; grad_out[3]: dJ/dvp, dJ/dvs, dJ/drho
 *   ([nz][pitch] each, may be NULL to skip), inside the box, 0 outside. */
int sgb_elastic_backward(const sgb_grid *grid, const sgb_elastic_model *model, const sgb_acquisition *acq,
                         const sgb_elastic_io *io, const sgb_bs_store *bs, float *const sbuf[10], int32_t scur,
                         float *const abuf[10], float *const grad_shot[3], const float *vp, const float *vs,
                         const float *rho, float *const grad_out[3], sgb_stream_t stream);

/* Chain rule of the elastic gradient terms: sums grad_shot[3] over shots and
 * maps the lambda / mu / buoyancy terms to dJ/dvp, dJ/dvs, dJ/drho
 * (grad_out entries may be NULL).  box != 0 restricts the result to the
 * interior box of bs (0 outside), as sgb_elastic_backward does. */
int sgb_elastic_gradient(const sgb_grid *grid, const sgb_elastic_model *model, const float *const grad_shot[3],
                         const float *vp, const float *vs, const float *rho, const sgb_bs_store *bs, int32_t box,
                         float *const grad_out[3], sgb_stream_t stream);

/* ------------------------------------------- misfit and post-processing --- */

/* L2 misfit of MSELoss(reduction='sum') summed over shots (loss.py:409-421):
 * *loss (device double, accumulated) += sum (syn - obs)^2 and, if resid is
 * not NULL, resid = 2 (syn - obs), the adjoint source. */
int sgb_l2_misfit(int64_t n, const float *syn, const float *obs, float *resid, double *loss,
                  sgb_stream_t stream);

/* out = grad (* mask) / (illum + eps) on [nz][pitch] planes (illum and mask
 * may be NULL): the gradient cut of process.py:43-47 and the illumination
 * preconditioning of process.py:115-118 (eps = 0 is the reference's plain
 * division); padding columns are written as 0. */
int sgb_grad_precondition(int32_t nz, int32_t nx, int32_t pitch, const float *grad, const float *illum,
                          float eps, const float *mask, float *out, sgb_stream_t stream);

/* `counts` passes of separable Gaussian smoothing, along z then x, in place
 * on grad (tmp: scratch of the same [nz][pitch] shape).  weights_* hold
 * 2 radius + 1 normalised taps; the boundary is numpy's 'reflect' padding
 * (signal.py:247-319, process.py:66-113). */
int sgb_grad_smooth(int32_t nz, int32_t nx, int32_t pitch, const float *weights_z, int32_t radius_z,
                    const float *weights_x, int32_t radius_x, int32_t counts, float *grad, float *tmp,
                    sgb_stream_t stream);

/* Steepest-descent step (optimizer.py:124-142): d = grad, clamped to
 * [lo, hi] when clamp != 0 (the reference's 2 % / 98 % quantiles, computed
 * by the caller), then param -= lr * d / max|d|.  scratch: one device
 * uint32. */
int sgb_sd_step(int64_t n, float *param, const float *grad, float lr, int32_t clamp, float lo, float hi,
                uint32_t *scratch, sgb_stream_t stream);

/* Non-linear conjugate-gradient step (optimizer.py:144-224, class Cg): d =
 * grad clamped to [lo, hi] when clamp != 0 (the caller's clip_value
 * quantiles); beta = (d - prev_grad) . d / |prev_grad|^2 (beta_type 0,
 * Polak-Ribiere) or |d|^2 / |prev_grad|^2 (1, Fletcher-Reeves), 0 while
 * prev_grad is all zero; direction = -d + beta direction; param += lr *
 * direction / max|direction|; prev_grad = d.  prev_grad starts at zeros.
 * scratch: 4 device doubles.  No host synchronisation. */
int sgb_ncg_step(int64_t n, float *param, const float *grad, float *prev_grad, float *direction, float lr,
                 int32_t beta_type, int32_t clamp, float lo, float hi, double *scratch, sgb_stream_t stream);

/* Zero-phase IIR filtering of records (scipy.signal.filtfilt with its
 * default odd padding, as SeisSignal.filter applies it to each shot,
 * signal.py:39-101): records [nt][ntraces] (trace fastest); b, a (a[0] = 1),
 * zi (lfilter_zi, ncoef - 1 values) are ncoef <= 17 device doubles; padlen
 * = 3 max(len a, len b), padlen < nt; work: [nt + 2 padlen][ntraces]
 * doubles.  out may alias in. */
int sgb_filtfilt(int32_t nt, int32_t ntraces, int32_t ncoef, const double *b, const double *a, const double *zi,
                 int32_t padlen, const float *in, float *out, double *work, sgb_stream_t stream);

/* --------------------------------------------- learned preconditioner --- */
/* BF16-weight / FP32-accumulate kernels of the convolutional gradient
 * preconditioner (no counterpart in the reference, which preconditions by
 * the illumination only, process.py:115-118).  Activations are bf16 NHWC
 * [n][h][w][c]; 3x3 convolutions with zero padding 1 run as implicit GEMMs
 * on the tcgen05 tensor cores (accumulator in tensor memory).  Channel
 * counts of tensor-core convolutions are multiples of 32; w is a multiple
 * of 64 (or 64 <= w < 128 with 128 % w == 0). */

/* y = conv3x3(x, wt) (+ bias) (ReLU) (* [mask > 0]), written to out_bf16
 * and/or out_f32 at [pixel * out_cstride + out_coff + co] (a channel slice
 * of a wider tensor, e.g. a skip concatenation).  wt: bf16 [cout][9][cin]
 * (tap = 3 ky + kx).  With wt flipped and transposed ([cin][9][cout], tap
 * 8 - t) the same call gives the data gradient. */
typedef struct {
  int32_t n, h, w, cin, cout;
  const void *x;
  const void *wt;
  const float *bias;  /* [cout] or NULL */
  int32_t relu;
  const void *mask;   /* bf16 NHWC or NULL */
  int32_t mask_cstride;
  void *out_bf16;     /* or NULL */
  float *out_f32;     /* or NULL */
  int32_t out_cstride, out_coff;
} sgb_nn_conv;
int sgb_nn_conv3x3(const sgb_nn_conv *c, sgb_stream_t stream);

/* dw[co][ci][tap] += sum over pixels of dy[co] * x[ci] at the tap's offset.
 * dy_chw: bf16 [n][cout][h][w]; x_chw[k]: bf16 [n][cin][h][w] holding the
 * input shifted by k - 1 columns (x_chw[k][..][x] = x[..][x - 1 + k], zero
 * outside), as sgb_nn_to_chw writes it; dw: fp32 [cout][cin][3][3]. */
typedef struct {
  int32_t n, h, w, cin, cout;
  const void *dy_chw;
  const void *x_chw[3];
  float *dw;
} sgb_nn_wgrad;
int sgb_nn_conv3x3_wgrad(const sgb_nn_wgrad *p, sgb_stream_t stream);

/* NHWC (channel slice [coff, coff + c) of a tensor with cstride channels)
 * -> CHW bf16 [copies][n][c][h][w]: copies = 1 gives the plain transpose,
 * copies = 3 the three column-shifted copies sgb_nn_conv3x3_wgrad reads. */
int sgb_nn_to_chw(int32_t n, int32_t h, int32_t w, int32_t c, int32_t cstride, int32_t coff, const void *x_nhwc,
                  int32_t copies, void *out, sgb_stream_t stream);

/* SIMT helpers of the network (h, w: the fine grid of the operation).
 * Input convolution: fp32 [n][2][h][w] -> c channels, ReLU; W [c][2][3][3].
 * Output convolution: c channels -> fp32 [n][h][w], linear; W [c][3][3].
 * Its backward writes dx (bf16 NHWC, c channels) times [act > 0] and
 * accumulates dW, db.  pool2: 2x2 average; up2: nearest 2x into a channel
 * slice; up2_bwd: 2x2 sums of a slice of an fp32 gradient times [act > 0];
 * pool2_bwd: gp / 4 (coarse, c channels) + an optional slice gs, times
 * [act > 0].  pack_weights: fp32 [cout][cin][3][3] -> bf16 [cout][9][cin]
 * and (if wflip) the flipped transpose [cin][9][cout] for data gradients.
 * bias_grad: db[c] += sum of a channel-major bf16 gradient [n][c][hw].
 * Channel counts, strides and offsets of these helpers are multiples of 8.
 * adam: one step (bias-corrected, step >= 1, decoupled weight decay wd).
 * mse: grad = 2 (pred - target) / n and *loss += mean squared error. */
int sgb_nn_conv_in(int32_t n, int32_t h, int32_t w, int32_t c, const float *in, const float *W, const float *b,
                   void *out, int32_t cstride, int32_t coff, sgb_stream_t stream);
int sgb_nn_conv_in_wgrad(int32_t n, int32_t h, int32_t w, int32_t c, const float *in, const void *dy,
                         int32_t dy_cstride, float *dW, float *db, sgb_stream_t stream);
int sgb_nn_conv_out(int32_t n, int32_t h, int32_t w, int32_t c, const void *in, int32_t cstride, const float *W,
                    const float *b, float *out, sgb_stream_t stream);
int sgb_nn_conv_out_bwd(int32_t n, int32_t h, int32_t w, int32_t c, const float *g, const float *W, const void *act,
                        int32_t act_cstride, void *dx, float *dW, float *db, sgb_stream_t stream);
int sgb_nn_pool2(int32_t n, int32_t h, int32_t w, int32_t c, const void *in, int32_t cs_in, int32_t coff_in,
                 void *out, sgb_stream_t stream);
int sgb_nn_up2(int32_t n, int32_t h, int32_t w, int32_t c, const void *in, void *out, int32_t cs_out,
               int32_t coff_out, sgb_stream_t stream);
int sgb_nn_up2_bwd(int32_t n, int32_t h, int32_t w, int32_t c, const float *g, int32_t cs_g, int32_t coff_g,
                   const void *act, void *out, sgb_stream_t stream);
int sgb_nn_pool2_bwd(int32_t n, int32_t h, int32_t w, int32_t c, const float *gp, const float *gs, int32_t cs_s,
                     int32_t coff_s, const void *act, int32_t cs_a, int32_t coff_a, void *out, sgb_stream_t stream);
int sgb_nn_bias_grad(int32_t n, int64_t hw, int32_t c, const void *dy_chw, float *db, sgb_stream_t stream);
int sgb_nn_pack_weights(int32_t cout, int32_t cin, const float *W, void *wt, void *wflip, sgb_stream_t stream);
int sgb_nn_adam(int64_t n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
                int32_t step, float wd, sgb_stream_t stream);
int sgb_nn_mse(int64_t n, const float *pred, const float *target, float *grad, float *loss, sgb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SEISTORCH_GB300_H */
