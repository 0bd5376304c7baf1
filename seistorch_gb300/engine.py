"""Host engine over the C ABI: pitched buffers, acquisition tables, time loops.

The hot path (every time step, source injection, receiver sampling, the
boundary ring, the adjoint) runs in the CUDA kernels of libseistorch_gb300;
this module only lays out device memory (torch tensors) and calls the C ABI
with raw pointers on the current torch stream.  There is no CPU path: calls
raise when CUDA or the library is unavailable.
"""
import ctypes
import math
import weakref

import numpy as np
import torch

from . import _native as N

BOUNDARY_PML = 0
BOUNDARY_HABC = 1


def pitch_of(nx):
    """Row stride (floats) of every device plane: nx rounded up to 4."""
    return (int(nx) + 3) // 4 * 4


def require_cuda(t, what):
    if not torch.cuda.is_available():
        raise RuntimeError(f"{what}: seistorch_gb300 needs a CUDA GPU (sm_103a); no CPU fallback")
    if t is not None and not t.is_cuda:
        raise RuntimeError(f"{what}: expected a CUDA tensor, got {t.device}")


_CFL_LAST = {}


def check_cfl(vel, scheme, order, dt, h, vmax_of=None):
    """Refuse a time step above the scheme's stability limit (sgb_cfl_check).

    ``vel`` is the model tensor the step depends on; ``vmax_of(vel)`` gives
    the effective maximum velocity (default: vel.max()).  The maximum is read
    once per tensor and version, so a per-step loop over the same model pays
    the device read once."""
    key = (scheme, int(order), float(dt), float(h))
    hit = _CFL_LAST.get(key)
    if hit is not None and hit[0]() is vel and hit[1] == vel._version:
        return
    vmax = float(vmax_of(vel)) if vmax_of is not None else float(vel.detach().max())
    N.cfl_check(scheme, order, vmax, dt, h)
    if len(_CFL_LAST) > 64:
        _CFL_LAST.clear()
    _CFL_LAST[key] = (weakref.ref(vel), vel._version)


def unpitched(t, nx):
    """The first nx columns of a pitched tensor as a tensor of its own (not a
    view), so callers may modify a step's output in place."""
    return t if t.shape[-1] == nx else t[..., :nx].contiguous()


def to_pitched(a, pitch, dtype=torch.float32):
    """(..., nz, nx) -> contiguous (..., nz, pitch) float32 with zero pad columns."""
    a = a.to(dtype)
    nx = a.shape[-1]
    if nx == pitch and a.is_contiguous():
        return a
    out = torch.zeros(*a.shape[:-1], pitch, dtype=dtype, device=a.device)
    out[..., :nx] = a
    return out


def grid_struct(nz, nx, pitch, nshots, dt, h):
    return N.Grid(int(nz), int(nx), int(pitch), int(nshots), float(dt), float(h))


class Acquisition:
    """Device tables for one batch of shots (rnn.py:158-212 semantics).

    sources:   per shot, a list of (z, x) padded-grid points; duplicates in a
               shot inject once (the 0/1 ``smask`` of rnn.py:158-166);
    src_wrow:  per shot, per point, the row of ``wavelet`` it injects
               (0 for the shared wavelet of the batched path);
    receivers: per shot, (zs, xs); records come back in the concatenated
               order of the shots (the super-probe order of rnn.py:51-73).
    """

    def __init__(self, nz, nx, sources, receivers, wavelet, device, src_wrow=None):
        nshots = len(sources)
        if len(receivers) != nshots:
            raise ValueError("sources and receivers must list the same number of shots")
        wav = torch.as_tensor(wavelet, dtype=torch.float32, device=device)
        if wav.ndim == 1:
            wav = wav[None]
        self.wavelet = wav.contiguous()
        self.nt = int(wav.shape[-1])
        sp, sz, sx, sw = [0], [], [], []
        for b, pts in enumerate(sources):
            seen = set()
            rows = src_wrow[b] if src_wrow is not None else [0] * len(pts)
            for (z, x), wr in zip(pts, rows):
                z, x = int(z), int(x)
                if not (0 <= z < nz and 0 <= x < nx):
                    raise IndexError(f"source ({z}, {x}) of shot {b} is outside the {nz}x{nx} grid")
                if (z, x) in seen:
                    continue
                seen.add((z, x))
                sz.append(z)
                sx.append(x)
                sw.append(int(wr))
            sp.append(len(sz))
        self.nshots = nshots
        self.nsrc = len(sz)
        if self.nsrc and max(sw) >= wav.shape[0]:
            raise IndexError("a source refers to a wavelet row that does not exist")
        it = lambda v: torch.as_tensor(np.asarray(v, np.int32), device=device)
        self.src_ptr, self.src_z, self.src_x, self.src_wrow = it(sp), it(sz), it(sx), it(sw)
        bz, zz, xx = [], [], []
        self.reccounts = []
        for b, (zs, xs) in enumerate(receivers):
            zs = np.asarray(zs, np.int64).reshape(-1)
            xs = np.asarray(xs, np.int64).reshape(-1)
            if zs.shape != xs.shape:
                raise ValueError(f"receiver z/x lists of shot {b} differ in length")
            if len(zs) and (zs.min() < 0 or zs.max() >= nz or xs.min() < 0 or xs.max() >= nx):
                raise IndexError(f"a receiver of shot {b} is outside the {nz}x{nx} grid")
            bz.append(np.full(len(zs), b, np.int64))
            zz.append(zs)
            xx.append(xs)
            self.reccounts.append(int(len(zs)))
        bz = np.concatenate(bz) if bz else np.zeros(0, np.int64)
        zz = np.concatenate(zz) if zz else np.zeros(0, np.int64)
        xx = np.concatenate(xx) if xx else np.zeros(0, np.int64)
        self.nrec = int(len(zz))
        key = (bz * nz + zz) * nx + xx
        order = np.argsort(key, kind="stable")
        row = (bz * nz + zz)[order]
        ptr = np.zeros(nshots * nz + 1, np.int64)
        np.add.at(ptr, row + 1, 1)
        ptr = np.cumsum(ptr)
        self.rec_row_ptr = it(ptr)
        self.rec_x = it(xx[order])
        self.rec_col = it(order)
        # per-shot [first, last+1) rows of sources and receivers
        szr = np.zeros((nshots, 2), np.int32)
        rzr = np.zeros((nshots, 2), np.int32)
        for b in range(nshots):
            zs_b = [int(z) for z in sz[sp[b]:sp[b + 1]]]
            if zs_b:
                szr[b] = (min(zs_b), max(zs_b) + 1)
        for b in range(nshots):
            zs_b = zz[bz == b]
            if len(zs_b):
                rzr[b] = (int(zs_b.min()), int(zs_b.max()) + 1)
        self.src_zr = it(szr)
        self.rec_zr = it(rzr)
        self.rec_b = torch.as_tensor(bz, device=device)
        self.rec_z = torch.as_tensor(zz, device=device)
        self.rec_xs = torch.as_tensor(xx, device=device)

    def with_wavelet(self, wavelet):
        """A copy with another wavelet (same number of rows) that shares this
        batch's source and receiver tables (a loop already in flight keeps
        its own wavelet)."""
        import copy
        wav = torch.as_tensor(wavelet, dtype=torch.float32, device=self.wavelet.device)
        if wav.ndim == 1:
            wav = wav[None]
        if wav.shape[0] != self.wavelet.shape[0]:
            raise ValueError("the new wavelet has a different number of rows")
        other = copy.copy(self)
        other.wavelet = wav.contiguous()
        other.nt = int(wav.shape[-1])
        return other

    def struct(self, records=None, nch=1):
        return N.Acquisition(
            N.ptr(self.src_ptr), N.ptr(self.src_z), N.ptr(self.src_x), N.ptr(self.src_wrow),
            N.ptr(self.wavelet), self.nsrc, self.nt,
            N.ptr(self.rec_row_ptr), N.ptr(self.rec_x), N.ptr(self.rec_col), self.nrec, int(nch),
            N.ptr(records), N.ptr(self.src_zr), N.ptr(self.rec_zr))


def interior_box(nz, nx, bwidth, multiple):
    """Undamped interior [iz0, iz1) x [ix0, ix1) of a padded grid."""
    top = 0 if multiple else bwidth
    return top, nz - bwidth, bwidth, nx - bwidth


class AcousticState:
    """Buffers one forward keeps for its adjoint."""

    def __init__(self):
        self.buf = None
        self.cur = 0
        self.prev = 1
        self.ring_store = None
        self.ckpt_store = None
        self.bs = None


class AcousticPropagator:
    """2nd-order acoustic time loop (acoustic.py / acoustic_habc.py + rnn.py)."""

    def __init__(self, nz, nx, dt, h, order=2, boundary="pml", bwidth=50, multiple=False,
                 device=None):
        if order not in (2, 4, 6, 8):
            raise ValueError(f"spatial order {order} is not supported (2, 4, 6 or 8)")
        self.nz, self.nx = int(nz), int(nx)
        self.pitch = pitch_of(nx)
        self.dt, self.h = float(dt), float(h)
        self.order = int(order)
        self.boundary = BOUNDARY_HABC if boundary == "habc" else BOUNDARY_PML
        self.bwidth = int(bwidth)
        self.multiple = bool(multiple)
        self.device = torch.device(device) if device is not None else torch.device("cuda")

    # -- coefficients
    def model(self, vp, damp, blend=True):
        """Pitched vp / damping planes and the (g, k) coefficient planes.
        ``blend=False`` (HABC only) drops the one-way blend: the plain
        undamped update of the reference's reverse steps."""
        require_cuda(vp, "AcousticPropagator.model")
        check_cfl(vp, N.SCHEME_ACOUSTIC, self.order, self.dt, self.h)
        vpp = to_pitched(vp.detach(), self.pitch).contiguous()
        dp = to_pitched(damp.detach().to(vp.device), self.pitch).contiguous()
        coef = torch.empty(2, self.nz, self.pitch, dtype=torch.float32, device=vp.device)
        g = grid_struct(self.nz, self.nx, self.pitch, 1, self.dt, self.h)
        N.call("sgb_acoustic_coefficients", ctypes.byref(g), N.ptr(vpp), N.ptr(dp), self.boundary,
               N.ptr(coef), N.stream_handle())
        m = N.AcousticModel(self.order, self.boundary, 50 if blend else 0, int(self.multiple), N.ptr(coef),
                            N.ptr(vpp), N.ptr(dp))
        return m, (vpp, dp, coef)

    def grid(self, nshots):
        return grid_struct(self.nz, self.nx, self.pitch, nshots, self.dt, self.h)

    # -- one step (equation-module drop-in)
    def step(self, vp, damp, u, um, blend=True):
        m, keep = self.model(vp, damp, blend)
        B = u.shape[0]
        up = to_pitched(u, self.pitch).contiguous()
        ump = to_pitched(um, self.pitch).contiguous()
        out = torch.empty_like(up)
        g = self.grid(B)
        N.call("sgb_acoustic_step", ctypes.byref(g), ctypes.byref(m), N.ptr(up), N.ptr(ump), N.ptr(out),
               N.stream_handle())
        return unpitched(out, self.nx)

    def step_vjp(self, vp, damp, u, gy, gh1):
        m, keep = self.model(vp, damp)
        B = u.shape[0]
        up = to_pitched(u, self.pitch).contiguous()
        gyp = to_pitched(gy, self.pitch).contiguous()
        gh1p = to_pitched(gh1, self.pitch).contiguous() if gh1 is not None else None
        gu = torch.empty_like(up)
        gum = torch.empty_like(up)
        gvp = torch.zeros(self.nz, self.pitch, dtype=torch.float32, device=up.device)
        g = self.grid(B)
        N.call("sgb_acoustic_step_vjp", ctypes.byref(g), ctypes.byref(m), N.ptr(up), N.ptr(gyp),
               N.ptr(gh1p), N.ptr(gu), N.ptr(gum), N.ptr(gvp), N.stream_handle())
        return gu[..., :self.nx], gum[..., :self.nx], gvp[:, :self.nx]

    def habc_vjp(self, m, u, um, gy, kz=None, rho_c=None, born=None, want_wi=False):
        """sgb_habc_step_vjp on pitched copies: dict of gu, gum (fields),
        gparam (1, 2 or 5 planes), gc (one-way velocity term) and, with
        ``born = (m plane, background U_n)``, born_gu and born_gm."""
        B = u.shape[0]
        pit = lambda t: to_pitched(t.to(torch.float32), self.pitch).contiguous()
        up, ump, gyp = pit(u), pit(um), pit(gy)
        dev = up.device
        out = {"gu": torch.empty_like(up), "gum": torch.empty_like(up),
               "gparam": torch.empty(5 if rho_c is not None else (2 if kz is not None else 1), self.nz,
                                     self.pitch, dtype=torch.float32, device=dev),
               "gc": torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev)}
        bm = bu = None
        if born is not None:
            bm = to_pitched(born[0].detach().to(device=dev, dtype=torch.float32), self.pitch).contiguous()
            bu = pit(born[1])
            out["born_gu"] = torch.empty_like(up)
            out["born_gm"] = torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev)
        if want_wi:
            out["wi"] = torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev)
        io = N.HabcVjpIO(N.ptr(up), N.ptr(ump), N.ptr(gyp), N.ptr(out["gu"]), N.ptr(out["gum"]),
                         N.ptr(out["gparam"]), N.ptr(out["gc"]), N.ptr(kz), N.ptr(rho_c), N.ptr(bm), N.ptr(bu),
                         N.ptr(out.get("born_gu")), N.ptr(out.get("born_gm")), N.ptr(out.get("wi")))
        g = self.grid(B)
        N.call("sgb_habc_step_vjp", ctypes.byref(g), ctypes.byref(m), ctypes.byref(io), N.stream_handle())
        nx = self.nx
        return {k: v[..., :nx] for k, v in out.items()}

    def step_vjp_habc(self, vp, damp, u, um, gy, blend=True):
        """VJP of one HABC step (acoustic_habc._time_step): dJ/du, dJ/dum and
        dJ/dvp over the whole grid (k = vp^2 dt^2 / h^2, so dk/dvp = 2 vp dt^2 / h^2)."""
        m, keep = self.model(vp, damp, blend)
        r = self.habc_vjp(m, u, um, gy)
        gvp = r["gparam"][0] * (2.0 * (self.dt / self.h) ** 2) * vp.detach().to(torch.float32)
        if blend:
            gvp = gvp + r["gc"]
        return r["gu"], r["gum"], gvp

    # -- whole loop
    def forward(self, vp, damp, acq, *, save_for_adjoint=False, illumination=False, ckpt_every=0,
                init=None):
        require_cuda(vp, "AcousticPropagator.forward")
        m, keep = self.model(vp, damp)
        B = acq.nshots
        dev = vp.device
        field = (B, self.nz, self.pitch)
        buf = [torch.zeros(field, dtype=torch.float32, device=dev) for _ in range(3)]
        if init is not None:
            buf[0][..., :self.nx] = init[0]
            buf[1][..., :self.nx] = init[1]
        records = torch.empty(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        illum = torch.zeros(self.nz, self.pitch, dtype=torch.float32, device=dev) if illumination else None
        state = AcousticState()
        bs_struct = None
        if save_for_adjoint:
            bs_struct = self._boundary_store(state, keep, B, acq.nt, ckpt_every, field, dev)
        cur = ctypes.c_int32(0)
        prev = ctypes.c_int32(0)
        g = self.grid(B)
        q = acq.struct(records if acq.nrec else None, 1)
        bufs = N.PTR3(*[b.data_ptr() for b in buf])
        N.call("sgb_acoustic_forward", ctypes.byref(g), ctypes.byref(m), ctypes.byref(q), bufs,
               N.ptr(illum), ctypes.byref(bs_struct) if bs_struct is not None else None,
               ctypes.byref(cur), ctypes.byref(prev), N.stream_handle())
        state.buf, state.cur, state.prev = buf, cur.value, prev.value
        state.keep = keep
        state.model = m
        return records[:, :acq.nrec], state, (illum[:, :self.nx] if illum is not None else None)

    def _boundary_store(self, state, keep, B, nt, ckpt_every, field, dev):
        """Ring store [nt][shots][ring] and checkpoints for the adjoint."""
        iz0, iz1, ix0, ix1 = interior_box(self.nz, self.nx, self.bwidth, self.multiple)
        if iz1 <= iz0 or ix1 <= ix0:
            raise ValueError("grid too small for its boundary width")
        dpl = keep[1][:, :self.nx]
        if torch.count_nonzero(dpl[iz0:iz1, ix0:ix1]).item() != 0:
            raise ValueError("the damping profile is not zero inside the interior box; "
                             "boundary-saving reconstruction needs an undamped interior")
        r = self.order // 2
        size = ctypes.c_int32(0)
        g1 = self.grid(B)
        N.call("sgb_ring_size", ctypes.byref(g1), iz0, iz1, ix0, ix1, r, ctypes.byref(size))
        state.ring_store = torch.empty(nt, B, max(size.value, 1), dtype=torch.float32, device=dev)
        K = int(ckpt_every) if ckpt_every else 0
        nslots = nt // K if K > 0 else 0
        state.ckpt_store = (torch.empty(max(nslots, 1), 2, *field, dtype=torch.float32, device=dev)
                            if K > 0 else None)
        # the HABC adjoints read each cell's static interior / side shares from five planes
        state.habc_planes = (torch.empty(5, self.nz, self.pitch, dtype=torch.float32, device=dev)
                             if self.boundary == BOUNDARY_HABC else None)
        state.bs = N.BsStore(iz0, iz1, ix0, ix1, r, size.value, N.ptr(state.ring_store), K,
                             N.ptr(state.ckpt_store), N.ptr(state.habc_planes))
        return state.bs

    def backward(self, state, acq, grad_records):
        """dJ/dvp (nz, nx) from dJ/d(records) through the fused adjoint."""
        B = acq.nshots
        dev = state.buf[0].device
        resid = torch.zeros(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        if acq.nrec:
            resid[:, :acq.nrec] = grad_records.to(torch.float32).reshape(acq.nt, acq.nrec, 1)
        field = (B, self.nz, self.pitch)
        lbuf = [torch.empty(field, dtype=torch.float32, device=dev) for _ in range(3)]
        grad_shot = torch.empty(field, dtype=torch.float32, device=dev)
        grad = torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev)
        g = self.grid(B)
        q = acq.struct(resid, 1)
        ub = N.PTR3(*[b.data_ptr() for b in state.buf])
        lb = N.PTR3(*[b.data_ptr() for b in lbuf])
        N.call("sgb_acoustic_backward", ctypes.byref(g), ctypes.byref(state.model), ctypes.byref(q),
               ctypes.byref(state.bs), ub, state.cur, state.prev, lb, N.ptr(grad_shot), N.ptr(grad),
               N.stream_handle())
        return grad[:, :self.nx]


class _AcousticLoop(torch.autograd.Function):
    """Whole acoustic time loop as one differentiable op: vp -> records."""

    @staticmethod
    def forward(ctx, vp, prop, damp, acq, illumination, ckpt_every):
        need = ctx.needs_input_grad[0]
        rec, state, illum = prop.forward(vp, damp, acq, save_for_adjoint=need, illumination=illumination,
                                         ckpt_every=ckpt_every)
        ctx.prop, ctx.acq, ctx.state = prop, acq, state
        ctx.mark_non_differentiable(illum) if illum is not None else None
        fields = (state.buf[state.cur][..., :prop.nx], state.buf[state.prev][..., :prop.nx])
        ctx.fields = fields
        return rec, illum if illum is not None else rec.new_zeros(0)

    @staticmethod
    def backward(ctx, grad_rec, grad_illum):
        if ctx.state.bs is None:
            return None, None, None, None, None, None
        grad_vp = ctx.prop.backward(ctx.state, ctx.acq, grad_rec.contiguous())
        ctx.state = None
        return grad_vp, None, None, None, None, None


def acoustic_loop(vp, prop, damp, acq, illumination=False, ckpt_every=0):
    """records (nt, nrec, 1) [, illum] of the acoustic loop; differentiable in vp."""
    rec, illum = _AcousticLoop.apply(vp, prop, damp, acq, illumination, ckpt_every)
    return rec, (illum if illumination else None)


def default_ckpt_every(nt):
    """Checkpoint spacing of the reconstruction: about sqrt(nt), at most 256."""
    return int(min(256, max(16, round(math.sqrt(max(nt, 1))))))


class BornPropagator(AcousticPropagator):
    """Born modelling of the acoustic HABC equation for least-squares RTM
    (acoustic_lsrtm_habc.py:11-30): a background field p driven by the
    sources and a scattered field s driven by m k L(p), both under the HABC
    blend; receivers sample s.  The gradient is dJ/dm (the velocity is held
    fixed, as in the reference's LSRTM configurations)."""

    def __init__(self, nz, nx, dt, h, order=2, bwidth=50, multiple=False, device=None):
        super().__init__(nz, nx, dt, h, order, "habc", bwidth, multiple, device)

    def forward_born(self, vp, refl, damp, acq, *, save_for_adjoint=False, ckpt_every=0):
        require_cuda(vp, "BornPropagator.forward_born")
        m, keep = self.model(vp, damp)
        B = acq.nshots
        dev = vp.device
        field = (B, self.nz, self.pitch)
        mp = to_pitched(refl.detach().to(device=dev, dtype=torch.float32), self.pitch).contiguous()
        pbuf = [torch.empty(field, dtype=torch.float32, device=dev) for _ in range(3)]
        sbuf = [torch.empty(field, dtype=torch.float32, device=dev) for _ in range(3)]
        src = torch.empty(field, dtype=torch.float32, device=dev)
        records = torch.empty(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        state = AcousticState()
        bs_struct = None
        if save_for_adjoint:
            bs_struct = self._boundary_store(state, keep, B, acq.nt, ckpt_every, field, dev)
        cur = ctypes.c_int32(0)
        prev = ctypes.c_int32(0)
        g = self.grid(B)
        q = acq.struct(records if acq.nrec else None, 1)
        N.call("sgb_born_forward", ctypes.byref(g), ctypes.byref(m), N.ptr(mp), ctypes.byref(q),
               N.PTR3(*[b.data_ptr() for b in pbuf]), N.PTR3(*[b.data_ptr() for b in sbuf]), N.ptr(src),
               ctypes.byref(bs_struct) if bs_struct is not None else None, ctypes.byref(cur), ctypes.byref(prev),
               N.stream_handle())
        state.buf, state.cur, state.prev = pbuf, cur.value, prev.value
        state.keep = keep
        state.model = m
        state.scattered = sbuf
        return records[:, :acq.nrec], state

    def step_vjp_born(self, vp, refl, damp, p, pm, sc, scm, gp, gs, blend=True):
        """VJP of one Born step (acoustic_lsrtm_habc._time_step) given dJ/dp+
        and dJ/ds+: dJ/d(p, pm, s, sm), dJ/dvp and dJ/dm."""
        m, keep = self.model(vp, damp, blend)
        rp = self.habc_vjp(m, p, pm, gp)
        rs = self.habc_vjp(m, sc, scm, gs, born=(refl, p))
        gvp = (rp["gparam"][0] + rs["gparam"][0]) * (2.0 * (self.dt / self.h) ** 2) * vp.detach().to(torch.float32)
        if blend:
            gvp = gvp + rp["gc"] + rs["gc"]
        return rp["gu"] + rs["born_gu"], rp["gum"], rs["gu"], rs["gum"], gvp, rs["born_gm"]

    def step_born(self, vp, refl, damp, p, pm, sc, scm, blend=True):
        """One step of both fields (no sources or receivers): (p+, s+)."""
        m, keep = self.model(vp, damp, blend)
        B = p.shape[0]
        pit = lambda t: to_pitched(t.to(torch.float32), self.pitch).contiguous()
        pp, ppm, ps, psm = pit(p), pit(pm), pit(sc), pit(scm)
        mp = to_pitched(refl.detach().to(device=p.device, dtype=torch.float32), self.pitch).contiguous()
        pn, sn, src = torch.empty_like(pp), torch.empty_like(pp), torch.empty_like(pp)
        g = self.grid(B)
        N.call("sgb_born_step", ctypes.byref(g), ctypes.byref(m), N.ptr(mp), N.ptr(pp), N.ptr(ppm), N.ptr(ps),
               N.ptr(psm), N.ptr(pn), N.ptr(sn), N.ptr(src), N.stream_handle())
        return unpitched(pn, self.nx), unpitched(sn, self.nx)

    def backward_born(self, state, acq, grad_records):
        """dJ/dm (nz, nx) from dJ/d(records) of the scattered field."""
        B = acq.nshots
        dev = state.buf[0].device
        resid = torch.zeros(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        if acq.nrec:
            resid[:, :acq.nrec] = grad_records.to(torch.float32).reshape(acq.nt, acq.nrec, 1)
        field = (B, self.nz, self.pitch)
        lbuf = [torch.empty(field, dtype=torch.float32, device=dev) for _ in range(3)]
        grad_shot = torch.empty(field, dtype=torch.float32, device=dev)
        grad = torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev)
        g = self.grid(B)
        q = acq.struct(resid, 1)
        N.call("sgb_born_backward", ctypes.byref(g), ctypes.byref(state.model), ctypes.byref(q),
               ctypes.byref(state.bs), N.PTR3(*[b.data_ptr() for b in state.buf]), state.cur, state.prev,
               N.PTR3(*[b.data_ptr() for b in lbuf]), N.ptr(grad_shot), N.ptr(grad), N.stream_handle())
        return grad[:, :self.nx]


class _BornLoop(torch.autograd.Function):
    """Whole Born loop as one differentiable op: reflectivity m -> records."""

    @staticmethod
    def forward(ctx, refl, vp, prop, damp, acq, ckpt_every):
        need = ctx.needs_input_grad[0]
        rec, state = prop.forward_born(vp, refl, damp, acq, save_for_adjoint=need, ckpt_every=ckpt_every)
        ctx.prop, ctx.acq, ctx.state = prop, acq, state
        return rec

    @staticmethod
    def backward(ctx, grad_rec):
        if ctx.state.bs is None:
            return None, None, None, None, None, None
        grad_m = ctx.prop.backward_born(ctx.state, ctx.acq, grad_rec.contiguous())
        ctx.state = None
        return grad_m, None, None, None, None, None


def born_loop(vp, refl, prop, damp, acq, ckpt_every=0):
    """Scattered-field records (nt, nrec, 1) of Born modelling; differentiable
    in the reflectivity ``refl`` (the background velocity is not)."""
    if vp.requires_grad:
        raise NotImplementedError("Born modelling differentiates the reflectivity m only "
                                  "(hold vp fixed, as the reference's LSRTM does)")
    return _BornLoop.apply(refl, vp.detach(), prop, damp, acq, ckpt_every)


def vti_coefficients(vp, eps, delta, dt, h):
    """x / z coefficient planes of vti_habc2._time_step (vti_habc2.py:26-51):
    sk = -2 (eps - delta) fx^2 fz^2 / ((1 + 2 eps) fx^4 + fz^4
    + 2 (1 + delta) fx^2 fz^2 + 1e-26) with fx / fz the FFT frequencies of
    the cell's row / column (torch.fft.fftfreq(n, d=h), as the reference's
    meshgrid), kx = vp^2 dt^2 (1 + 2 eps + sk) / h^2, kz = vp^2 dt^2 (1 + sk) / h^2.
    Differentiable in vp, eps and delta (the adjoint's chain rule)."""
    nz, nx = vp.shape[-2:]
    dev = vp.device
    fx = torch.fft.fftfreq(nz, d=float(h), dtype=torch.float64, device=dev)
    fz = torch.fft.fftfreq(nx, d=float(h), dtype=torch.float64, device=dev)
    fxx, fzz = torch.meshgrid(fx, fz, indexing="ij")
    vp, eps, delta = vp.double(), eps.double(), delta.double()
    num = -2.0 * (eps - delta) * fxx ** 2 * fzz ** 2
    den = (1.0 + 2.0 * eps) * fxx ** 4 + fzz ** 4 + 2.0 * (1.0 + delta) * fxx ** 2 * fzz ** 2
    sk = num * (den + 1e-26) ** -1
    v2 = vp ** 2 * float(dt) ** 2 / float(h) ** 2
    return v2 * ((1.0 + 2.0 * eps) + sk), v2 * (1.0 + sk)


class VTIPropagator(AcousticPropagator):
    """VTI acoustic equation with the HABC (vti_habc2.py), 2nd order."""

    def __init__(self, nz, nx, dt, h, bwidth=50, multiple=False, device=None):
        super().__init__(nz, nx, dt, h, 2, "habc", bwidth, multiple, device)

    def model_vti(self, vp, eps, delta, damp, blend=True):
        require_cuda(vp, "VTIPropagator.model_vti")
        cx, cz = vti_coefficients(vp.detach(), eps.detach(), delta.detach(), self.dt, self.h)
        # stability of 2u - u- + kx Lx + kz Lz: the isotropic limit with the
        # velocity sqrt((kx + kz) / 2) h / dt
        check_cfl(vp, N.SCHEME_ACOUSTIC, 2, self.dt, self.h,
                  lambda _: float(((cx + cz) / 2).clamp_min(0).max().sqrt()) * self.h / self.dt)
        coef = torch.empty(3, self.nz, self.pitch, dtype=torch.float32, device=vp.device)
        coef[0] = 2.0
        coef[1] = to_pitched(cx.float(), self.pitch)
        coef[2] = to_pitched(cz.float(), self.pitch)
        vpp = to_pitched(vp.detach().float(), self.pitch).contiguous()
        dp = to_pitched(damp.detach().to(vp.device).float(), self.pitch).contiguous()
        m = N.AcousticModel(2, BOUNDARY_HABC, 50 if blend else 0, int(self.multiple), N.ptr(coef), N.ptr(vpp),
                            N.ptr(dp))
        return m, (vpp, dp, coef)

    def step_vjp_vti(self, vp, eps, delta, damp, u, um, gy, blend=True):
        """VJP of one VTI step (vti_habc2._time_step): dJ/du, dJ/dum and
        dJ/d(vp, eps, delta), the coefficient planes' terms mapped through
        the differentiable coefficient map."""
        m, keep = self.model_vti(vp, eps, delta, damp, blend)
        r = self.habc_vjp(m, u, um, gy, kz=keep[2][2])
        with torch.enable_grad():
            ins = [t.detach().requires_grad_(True) for t in (vp, eps, delta)]
            cx, cz = vti_coefficients(*ins, self.dt, self.h)
            grads = torch.autograd.grad((cx, cz), ins, (r["gparam"][0].double(), r["gparam"][1].double()),
                                        allow_unused=True)
        grads = [torch.zeros_like(t, dtype=torch.float64) if g_ is None else g_ for g_, t in zip(grads, ins)]
        if blend:
            grads[0] = grads[0] + r["gc"].double()
        return r["gu"], r["gum"], grads

    def step_vti(self, vp, eps, delta, damp, u, um, blend=True):
        m, keep = self.model_vti(vp, eps, delta, damp, blend)
        up = to_pitched(u.float(), self.pitch).contiguous()
        ump = to_pitched(um.float(), self.pitch).contiguous()
        out = torch.empty_like(up)
        g = self.grid(u.shape[0])
        N.call("sgb_vti_step", ctypes.byref(g), ctypes.byref(m), N.ptr(up), N.ptr(ump), N.ptr(out),
               N.stream_handle())
        return unpitched(out, self.nx)

    def forward_vti(self, vp, eps, delta, damp, acq, *, save_for_adjoint=False, ckpt_every=0):
        m, keep = self.model_vti(vp, eps, delta, damp)
        B = acq.nshots
        dev = vp.device
        field = (B, self.nz, self.pitch)
        buf = [torch.zeros(field, dtype=torch.float32, device=dev) for _ in range(3)]
        records = torch.empty(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        state = AcousticState()
        bs_struct = None
        if save_for_adjoint:
            bs_struct = self._boundary_store(state, keep, B, acq.nt, ckpt_every, field, dev)
        cur = ctypes.c_int32(0)
        prev = ctypes.c_int32(0)
        g = self.grid(B)
        q = acq.struct(records if acq.nrec else None, 1)
        N.call("sgb_vti_forward", ctypes.byref(g), ctypes.byref(m), ctypes.byref(q),
               N.PTR3(*[b.data_ptr() for b in buf]), ctypes.byref(bs_struct) if bs_struct is not None else None,
               ctypes.byref(cur), ctypes.byref(prev), N.stream_handle())
        state.buf, state.cur, state.prev = buf, cur.value, prev.value
        state.keep = keep
        state.model = m
        return records[:, :acq.nrec], state

    def backward_vti(self, state, acq, grad_records):
        """(dJ/dkx, dJ/dkz) planes (nz, nx) from dJ/d(records)."""
        B = acq.nshots
        dev = state.buf[0].device
        resid = torch.zeros(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        if acq.nrec:
            resid[:, :acq.nrec] = grad_records.to(torch.float32).reshape(acq.nt, acq.nrec, 1)
        field = (B, self.nz, self.pitch)
        lbuf = [torch.empty(field, dtype=torch.float32, device=dev) for _ in range(3)]
        gsx, gsz = torch.empty(field, dtype=torch.float32, device=dev), torch.empty(field, dtype=torch.float32, device=dev)
        gx = torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev)
        gz = torch.empty_like(gx)
        g = self.grid(B)
        q = acq.struct(resid, 1)
        N.call("sgb_vti_backward", ctypes.byref(g), ctypes.byref(state.model), ctypes.byref(q),
               ctypes.byref(state.bs), N.PTR3(*[b.data_ptr() for b in state.buf]), state.cur, state.prev,
               N.PTR3(*[b.data_ptr() for b in lbuf]), N.ptr(gsx), N.ptr(gsz), N.ptr(gx), N.ptr(gz),
               N.stream_handle())
        return gx[:, :self.nx], gz[:, :self.nx]


class _VTILoop(torch.autograd.Function):
    """Whole VTI loop as one differentiable op: (vp, eps, delta) -> records."""

    @staticmethod
    def forward(ctx, vp, eps, delta, prop, damp, acq, ckpt_every):
        need = any(ctx.needs_input_grad[:3])
        rec, state = prop.forward_vti(vp, eps, delta, damp, acq, save_for_adjoint=need, ckpt_every=ckpt_every)
        ctx.prop, ctx.acq, ctx.state = prop, acq, state
        ctx.save_for_backward(vp, eps, delta)
        return rec

    @staticmethod
    def backward(ctx, grad_rec):
        if ctx.state.bs is None:
            return (None,) * 7
        gx, gz = ctx.prop.backward_vti(ctx.state, ctx.acq, grad_rec.contiguous())
        ctx.state = None
        vp, eps, delta = ctx.saved_tensors
        with torch.enable_grad():
            ins = [t.detach().requires_grad_(True) for t in (vp, eps, delta)]
            cx, cz = vti_coefficients(*ins, ctx.prop.dt, ctx.prop.h)
            grads = torch.autograd.grad((cx, cz), ins, (gx.double(), gz.double()), allow_unused=True)
        out = [None if g_ is None else g_.to(t.dtype) for g_, t in zip(grads, (vp, eps, delta))]
        return out[0], out[1], out[2], None, None, None, None


def vti_loop(vp, eps, delta, prop, damp, acq, ckpt_every=0):
    """Records (nt, nrec, 1) of the VTI loop; differentiable in vp, eps, delta."""
    return _VTILoop.apply(vp, eps, delta, prop, damp, acq, ckpt_every)


def rho_coefficients(vp, rho, dt, h):
    """Five planes of acoustic_rho_habc._time_step (acoustic_rho_habc.py:34-58):
    C = dt^2 rho vp^2 / h^2 and the buoyancy averages bx+, bx-, bz+, bz- of
    b = 1 / rho ((b + b[x+1]) / 2 ... with zeros beyond the grid, the
    reference's zero-padded convolutions).  Differentiable in vp and rho."""
    vp, rho = vp.double(), rho.double()
    b = 1.0 / rho
    bp = torch.nn.functional.pad(b, (1, 1, 1, 1))
    bxp = (b + bp[1:-1, 2:]) / 2
    bxn = (bp[1:-1, :-2] + b) / 2
    bzp = (b + bp[2:, 1:-1]) / 2
    bzn = (bp[:-2, 1:-1] + b) / 2
    C = float(dt) ** 2 / float(h) ** 2 * rho * vp ** 2
    return C, bxp, bxn, bzp, bzn


class RhoPropagator(AcousticPropagator):
    """Variable-density acoustic equation with the HABC (acoustic_rho_habc.py),
    2nd order."""

    def __init__(self, nz, nx, dt, h, bwidth=50, multiple=False, device=None):
        super().__init__(nz, nx, dt, h, 2, "habc", bwidth, multiple, device)

    def planes(self, vp, rho):
        planes = rho_coefficients(vp.detach(), rho.detach(), self.dt, self.h)
        out = torch.empty(5, self.nz, self.pitch, dtype=torch.float32, device=vp.device)
        for i, p_ in enumerate(planes):
            out[i] = to_pitched(p_.float(), self.pitch)
        return out

    def step_vjp_rho(self, vp, rho, damp, u, um, gy, blend=True):
        """VJP of one variable-density step (acoustic_rho_habc._time_step):
        dJ/du, dJ/dum and dJ/d(vp, rho) through the differentiable planes."""
        m, keep = self.model(vp, damp, blend)
        rc = self.planes(vp, rho)
        r = self.habc_vjp(m, u, um, gy, rho_c=rc)
        with torch.enable_grad():
            ins = [t.detach().requires_grad_(True) for t in (vp, rho)]
            planes = rho_coefficients(*ins, self.dt, self.h)
            grads = torch.autograd.grad(planes, ins, [r["gparam"][q].double() for q in range(5)], allow_unused=True)
        grads = [torch.zeros_like(t, dtype=torch.float64) if g_ is None else g_ for g_, t in zip(grads, ins)]
        if blend:
            grads[0] = grads[0] + r["gc"].double()
        return r["gu"], r["gum"], grads

    def step_rho(self, vp, rho, damp, u, um, blend=True):
        m, keep = self.model(vp, damp, blend)
        rc = self.planes(vp, rho)
        up = to_pitched(u.float(), self.pitch).contiguous()
        ump = to_pitched(um.float(), self.pitch).contiguous()
        out = torch.empty_like(up)
        g = self.grid(u.shape[0])
        N.call("sgb_rho_step", ctypes.byref(g), ctypes.byref(m), N.ptr(rc), N.ptr(up), N.ptr(ump), N.ptr(out),
               N.stream_handle())
        return unpitched(out, self.nx)

    def forward_rho(self, vp, rho, damp, acq, *, save_for_adjoint=False, ckpt_every=0):
        m, keep = self.model(vp, damp)
        rc = self.planes(vp, rho)
        B = acq.nshots
        dev = vp.device
        field = (B, self.nz, self.pitch)
        buf = [torch.zeros(field, dtype=torch.float32, device=dev) for _ in range(3)]
        records = torch.empty(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        state = AcousticState()
        bs_struct = None
        if save_for_adjoint:
            bs_struct = self._boundary_store(state, keep, B, acq.nt, ckpt_every, field, dev)
        cur = ctypes.c_int32(0)
        prev = ctypes.c_int32(0)
        g = self.grid(B)
        q = acq.struct(records if acq.nrec else None, 1)
        N.call("sgb_rho_forward", ctypes.byref(g), ctypes.byref(m), N.ptr(rc), ctypes.byref(q),
               N.PTR3(*[b.data_ptr() for b in buf]), ctypes.byref(bs_struct) if bs_struct is not None else None,
               ctypes.byref(cur), ctypes.byref(prev), N.stream_handle())
        state.buf, state.cur, state.prev = buf, cur.value, prev.value
        state.keep = (keep, rc)
        state.model = m
        state.rho_c = rc
        return records[:, :acq.nrec], state

    def backward_rho(self, state, acq, grad_records):
        """The five coefficient gradients (5, nz, nx) from dJ/d(records)."""
        B = acq.nshots
        dev = state.buf[0].device
        resid = torch.zeros(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        if acq.nrec:
            resid[:, :acq.nrec] = grad_records.to(torch.float32).reshape(acq.nt, acq.nrec, 1)
        field = (B, self.nz, self.pitch)
        lbuf = [torch.empty(field, dtype=torch.float32, device=dev) for _ in range(3)]
        gshot = torch.empty(5, *field, dtype=torch.float32, device=dev)
        grad = torch.empty(5, self.nz, self.pitch, dtype=torch.float32, device=dev)
        g = self.grid(B)
        q = acq.struct(resid, 1)
        N.call("sgb_rho_backward", ctypes.byref(g), ctypes.byref(state.model), N.ptr(state.rho_c), ctypes.byref(q),
               ctypes.byref(state.bs), N.PTR3(*[b.data_ptr() for b in state.buf]), state.cur, state.prev,
               N.PTR3(*[b.data_ptr() for b in lbuf]), N.ptr(gshot), N.ptr(grad), N.stream_handle())
        return grad[:, :, :self.nx]


class _RhoLoop(torch.autograd.Function):
    """Whole variable-density loop as one differentiable op: (vp, rho) -> records."""

    @staticmethod
    def forward(ctx, vp, rho, prop, damp, acq, ckpt_every):
        need = any(ctx.needs_input_grad[:2])
        rec, state = prop.forward_rho(vp, rho, damp, acq, save_for_adjoint=need, ckpt_every=ckpt_every)
        ctx.prop, ctx.acq, ctx.state = prop, acq, state
        ctx.save_for_backward(vp, rho)
        return rec

    @staticmethod
    def backward(ctx, grad_rec):
        if ctx.state.bs is None:
            return (None,) * 6
        g5 = ctx.prop.backward_rho(ctx.state, ctx.acq, grad_rec.contiguous())
        ctx.state = None
        vp, rho = ctx.saved_tensors
        with torch.enable_grad():
            ins = [t.detach().requires_grad_(True) for t in (vp, rho)]
            planes = rho_coefficients(*ins, ctx.prop.dt, ctx.prop.h)
            grads = torch.autograd.grad(planes, ins, [g.double() for g in g5], allow_unused=True)
        # defined inside the undamped box (the rim terms only complete the
        # box's edge cells), 0 outside, as the other adjoints
        iz0, iz1, ix0, ix1 = interior_box(ctx.prop.nz, ctx.prop.nx, ctx.prop.bwidth, ctx.prop.multiple)
        box = torch.zeros_like(vp, dtype=torch.bool)
        box[iz0:iz1, ix0:ix1] = True
        out = [None if g_ is None else torch.where(box, g_, 0.0).to(t.dtype) for g_, t in zip(grads, (vp, rho))]
        return out[0], out[1], None, None, None, None


def rho_loop(vp, rho, prop, damp, acq, ckpt_every=0):
    """Records (nt, nrec, 1) of the variable-density loop; differentiable in vp and rho."""
    return _RhoLoop.apply(vp, rho, prop, damp, acq, ckpt_every)


def vacoustic_coefficients(vp, Q, dt, h, omega=16.5):
    """Planes of vacoustic_habc._time_step (vacoustic_habc.py:74-111): the
    Laplacian coefficient kv = vp^2 dt^2 (1 - (1 - sqrt(Q^2 + 1)) / Q^2) / h^2
    (wave term plus phase correction) and the damping coefficient
    a_neg = -dt t vp / 2 of K(U - U-) with t_sigma = (sqrt(1 + Q^-2) - 1/Q) /
    omega, t_eps = 1 / (omega^2 t_sigma), t = t_eps / (t_sigma - 1e-8) - 1.
    The reference uses omega = 16.5 in its forward step and 5.0 in its
    reverse steps.  Differentiable in vp and Q (float64)."""
    vp, Q = vp.double(), Q.double()
    t_sigma = (torch.sqrt(1.0 + Q ** -2) - Q ** -1) / omega
    t_eps = (omega ** 2 * t_sigma) ** -1
    t = t_eps / (t_sigma - 1e-8) - 1.0
    kv = vp ** 2 * float(dt) ** 2 / float(h) ** 2 * (1.0 - (1.0 - torch.sqrt(Q ** 2 + 1.0)) * Q ** -2)
    return kv, -(float(dt) * t * vp / 2.0)


class VacousticPropagator(AcousticPropagator):
    """Viscoacoustic equation with the HABC (vacoustic_habc.py): the acoustic
    HABC step with the Laplacian coefficient kv and the spectral damping term
    a_neg K(U - U-), K = real(ifft2(|k| fft2(.))) (sgb_vacoustic_kterm)."""

    def __init__(self, nz, nx, dt, h, order=2, bwidth=50, multiple=False, device=None):
        super().__init__(nz, nx, dt, h, order, "habc", bwidth, multiple, device)

    def model_vac(self, vp, Q, damp, blend=True, omega=16.5):
        require_cuda(vp, "VacousticPropagator.model_vac")
        kv, an = vacoustic_coefficients(vp.detach(), Q.detach(), self.dt, self.h, omega)
        check_cfl(vp, N.SCHEME_ACOUSTIC, self.order, self.dt, self.h,
                  lambda _: float(kv.clamp_min(0).max().sqrt()) * self.h / self.dt)
        coef = torch.empty(2, self.nz, self.pitch, dtype=torch.float32, device=vp.device)
        coef[0] = 2.0
        coef[1] = to_pitched(kv.float(), self.pitch)
        a_neg = to_pitched(an.float(), self.pitch).contiguous()
        vpp = to_pitched(vp.detach().float(), self.pitch).contiguous()
        dp = to_pitched(damp.detach().to(vp.device).float(), self.pitch).contiguous()
        m = N.AcousticModel(self.order, BOUNDARY_HABC, 50 if blend else 0, int(self.multiple), N.ptr(coef), N.ptr(vpp),
                            N.ptr(dp))
        return m, (vpp, dp, coef, a_neg)

    def scratch(self, nshots, dev):
        g = self.grid(nshots)
        wf, tf = ctypes.c_int64(0), ctypes.c_int64(0)
        N.call("sgb_vacoustic_work_size", ctypes.byref(g), ctypes.byref(wf), ctypes.byref(tf))
        return (torch.empty(wf.value, dtype=torch.float32, device=dev),
                torch.empty(tf.value, dtype=torch.float32, device=dev))

    def kterm(self, u1, u2=None, pre=None, post=None):
        """post * K(pre * (u1 - u2)) per shot (pitched planes / fields)."""
        B = u1.shape[0]
        work, tw = self.scratch(B, u1.device)
        out = torch.empty_like(u1)
        g = self.grid(B)
        N.call("sgb_vacoustic_kterm", ctypes.byref(g), N.ptr(pre), N.ptr(u1), N.ptr(u2), N.ptr(post), N.ptr(out),
               N.ptr(work), N.ptr(tw), N.stream_handle())
        return out

    def step_vac(self, vp, Q, damp, u, um, blend=True, omega=16.5):
        m, keep = self.model_vac(vp, Q, damp, blend, omega)
        pit = lambda t: to_pitched(t.to(torch.float32), self.pitch).contiguous()
        up, ump = pit(u), pit(um)
        out, extra = torch.empty_like(up), torch.empty_like(up)
        work, tw = self.scratch(u.shape[0], up.device)
        g = self.grid(u.shape[0])
        N.call("sgb_vacoustic_step", ctypes.byref(g), ctypes.byref(m), N.ptr(keep[3]), N.ptr(up), N.ptr(ump),
               N.ptr(out), N.ptr(extra), N.ptr(work), N.ptr(tw), N.stream_handle())
        return unpitched(out, self.nx)

    def step_vjp_vac(self, vp, Q, damp, u, um, gy, blend=True, omega=16.5):
        """VJP of one step: dJ/du, dJ/dum, dJ/d(vp, Q).  The blended interior
        update wi (2u - um + kv L(u) + a_neg K(u - um)) + one-way terms: the
        HABC transposes (sgb_habc_step_vjp) plus K(a_neg wi gy) (K is
        symmetric) into dJ/du and minus it into dJ/dum, and
        dJ/da_neg = sum_b wi gy K(u - um)."""
        m, keep = self.model_vac(vp, Q, damp, blend, omega)
        r = self.habc_vjp(m, u, um, gy, want_wi=True)
        pit = lambda t: to_pitched(t.to(torch.float32), self.pitch).contiguous()
        wi = to_pitched(r["wi"], self.pitch).contiguous()
        F = self.kterm(pit(gy), pre=(keep[3] * wi).contiguous())[..., :self.nx]
        Kd = self.kterm(pit(u), pit(um))[..., :self.nx]
        g_an = (r["wi"][None] * gy.to(torch.float32) * Kd).sum(0)
        with torch.enable_grad():
            ins = [t.detach().requires_grad_(True) for t in (vp, Q)]
            kv, an = vacoustic_coefficients(*ins, self.dt, self.h, omega)
            grads = torch.autograd.grad((kv, an), ins, (r["gparam"][0].double(), g_an.double()), allow_unused=True)
        grads = [torch.zeros_like(t, dtype=torch.float64) if g_ is None else g_ for g_, t in zip(grads, ins)]
        if blend:
            grads[0] = grads[0] + r["gc"].double()
        return r["gu"] + F, r["gum"] - F, grads

    def forward_vac(self, vp, Q, damp, acq):
        """Records (nt, nrec, 1) of the whole loop (no adjoint state)."""
        m, keep = self.model_vac(vp, Q, damp)
        B = acq.nshots
        dev = vp.device
        field = (B, self.nz, self.pitch)
        buf = [torch.zeros(field, dtype=torch.float32, device=dev) for _ in range(3)]
        extra = torch.empty(field, dtype=torch.float32, device=dev)
        work, tw = self.scratch(B, dev)
        records = torch.empty(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=dev)
        cur, prev = ctypes.c_int32(0), ctypes.c_int32(0)
        g = self.grid(B)
        q = acq.struct(records if acq.nrec else None, 1)
        N.call("sgb_vacoustic_forward", ctypes.byref(g), ctypes.byref(m), N.ptr(keep[3]), ctypes.byref(q),
               N.PTR3(*[b_.data_ptr() for b_ in buf]), N.ptr(extra), N.ptr(work), N.ptr(tw), ctypes.byref(cur),
               ctypes.byref(prev), N.stream_handle())
        self._last = (buf, cur.value, prev.value)
        return records[:, :acq.nrec]


class VacousticStep(torch.autograd.Function):
    """One native viscoacoustic step with its native VJP (the per-step op of
    vacoustic_habc._time_step and of its reverse steps)."""

    @staticmethod
    def forward(ctx, vp, Q, h1, h2, damp, prop, blend, omega):
        ctx.prop, ctx.blend, ctx.omega = prop, blend, omega
        ctx.save_for_backward(vp, Q, h1, h2, damp)
        return prop.step_vac(vp, Q, damp, h1, h2, blend, omega)

    @staticmethod
    def backward(ctx, gy):
        vp, Q, h1, h2, damp = ctx.saved_tensors
        gu, gum, gm = ctx.prop.step_vjp_vac(vp, Q, damp, h1, h2, gy.contiguous().to(torch.float32), ctx.blend,
                                            ctx.omega)
        return (gm[0].to(vp.dtype), gm[1].to(Q.dtype), gu.to(h1.dtype), gum.to(h2.dtype), None, None, None, None)


def vacoustic_records(vp, Q, prop, damp, acq):
    """Records (nt, nrec, 1) of the viscoacoustic loop.  Without gradients:
    the native whole loop (sgb_vacoustic_forward).  With gradients: the loop
    step by step under autograd (native steps and VJPs), which is what the
    reference differentiates -- its spectral damping term has no explicit
    time reversal, so no boundary-saving reconstruction applies."""
    if not (torch.is_grad_enabled() and (vp.requires_grad or Q.requires_grad)):
        with torch.no_grad():
            return prop.forward_vac(vp, Q, damp, acq)
    B, dev = acq.nshots, vp.device
    sp = acq.src_ptr.cpu().tolist()
    sb = torch.as_tensor(np.repeat(np.arange(B), np.diff(sp)), device=dev)
    sz, sx, sw = acq.src_z.long(), acq.src_x.long(), acq.src_wrow.long()
    h1 = torch.zeros(B, prop.nz, prop.nx, device=dev)
    h2 = torch.zeros_like(h1)
    recs = []
    for t in range(acq.nt):
        y = VacousticStep.apply(vp, Q, h1, h2, damp, prop, True, 16.5)
        if acq.nsrc:
            y = y.index_put((sb, sz, sx), acq.wavelet[sw, t], accumulate=True)
        h2, h1 = h1, y
        recs.append(y[acq.rec_b, acq.rec_z, acq.rec_xs])
    return torch.stack(recs)[..., None]


class UnevenBatch:
    """Acoustic PML time loops of several grids (different shapes, shots and
    trace lengths) run together: one persistent launch per step covers the
    tiles of every grid still running (``sgb_acoustic_batch_forward``), and
    ``plan()`` records the whole loop once as a CUDA graph that ``replay()``
    relaunches with a single call.

    groups: list of (AcousticPropagator, vp (nz, nx), damping (nz, nx),
    Acquisition); every propagator must use the same spatial order.
    """

    MAX_GROUPS = 8

    def __init__(self, groups):
        if not 1 <= len(groups) <= self.MAX_GROUPS:
            raise ValueError(f"an uneven batch holds 1 to {self.MAX_GROUPS} grids")
        orders = {p.order for p, _, _, _ in groups}
        if len(orders) != 1:
            raise ValueError("every grid of an uneven batch must use the same spatial order")
        self.groups = groups
        self._keep = []
        structs = []
        self.records = []
        self.buffers = []
        for prop, vp, damp, acq in groups:
            require_cuda(vp, "UnevenBatch")
            if prop.boundary != BOUNDARY_PML:
                raise NotImplementedError("the uneven batch covers the PML acoustic equation")
            m, keep = prop.model(vp, damp)
            B = acq.nshots
            buf = [torch.zeros(B, prop.nz, prop.pitch, dtype=torch.float32, device=vp.device) for _ in range(3)]
            rec = torch.zeros(acq.nt, max(acq.nrec, 1), 1, dtype=torch.float32, device=vp.device)
            q = acq.struct(rec if acq.nrec else None, 1)
            structs.append(N.BatchGroup(prop.grid(B), m, q, N.PTR3(*[b.data_ptr() for b in buf]), None))
            self._keep.append((keep, buf, rec, acq))
            self.records.append(rec)
            self.buffers.append(buf)
        self._arr = (N.BatchGroup * len(structs))(*structs)
        self.cur = (ctypes.c_int32 * len(structs))()
        self.prev = (ctypes.c_int32 * len(structs))()
        self._plan = None

    def points(self):
        """Grid-point updates of one run: sum over grids of shots * nz * nx * nt."""
        return sum(acq.nshots * p.nz * p.nx * acq.nt for p, _, _, acq in self.groups)

    def run(self):
        N.call("sgb_acoustic_batch_forward", self._arr, len(self.groups), self.cur, self.prev,
               N.stream_handle())
        return self.result()

    def plan(self):
        if self._plan is None:
            h = ctypes.c_void_p(None)
            N.call("sgb_acoustic_batch_plan", self._arr, len(self.groups), self.cur, self.prev, ctypes.byref(h))
            self._plan = h
        return self

    def replay(self):
        if self._plan is None:
            self.plan()
        N.call("sgb_plan_launch", self._plan, N.stream_handle())
        return self.result()

    def result(self):
        """Per grid: records (nt, nrec, 1)."""
        return [r[:, :acq.nrec] for r, (_, _, _, acq) in zip(self.records, self.groups)]

    def close(self):
        if self._plan is not None:
            N.load().sgb_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
