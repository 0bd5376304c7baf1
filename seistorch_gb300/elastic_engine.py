"""Host engine of the isotropic elastic velocity-stress path (elastic.py:7-37).

Lays out the five pitched fields per shot, the coefficient planes and the
boundary-saving store, and calls the elastic entry points of the C ABI on the
current torch stream.  The whole time loop is one differentiable op in
(vp, vs, rho): its backward is the fused reverse kernel (reconstruction of
the forward state inside the undamped box from a one-cell ring + checkpoints,
exact discrete adjoint, gradient terms), replacing checkpoint.py:108-230.
"""
import ctypes

import torch

from . import _native as N
from .engine import check_cfl, grid_struct, interior_box, pitch_of, require_cuda, to_pitched, unpitched

FIELDS = ("vx", "vz", "txx", "tzz", "txz")  # Wavefield('elastic') order (eqconfigure.py:45-127)


def field_index(name):
    try:
        return FIELDS.index(name)
    except ValueError:
        raise ValueError(f"'{name}' is not an elastic wavefield ({', '.join(FIELDS)})") from None


def make_io(source_type, receiver_type):
    """sgb_elastic_io from the config's source_type / receiver_type lists."""
    source_type = list(source_type or ["txx", "tzz"])
    receiver_type = list(receiver_type or ["vx", "vz"])
    if not 1 <= len(receiver_type) <= 4:
        raise ValueError("elastic receivers record 1 to 4 wavefields")
    mask = 0
    for s in source_type:
        mask |= 1 << field_index(s)
    rec = (ctypes.c_int32 * 4)(*([field_index(r) for r in receiver_type] + [0] * (4 - len(receiver_type))))
    return N.ElasticIO(mask, rec, field_index(source_type[-1])), len(receiver_type)


class ElasticState:
    """Buffers one forward keeps for its adjoint."""

    def __init__(self):
        self.buf = None
        self.cur = 0
        self.ring_store = None
        self.ckpt_store = None
        self.bs = None
        self.keep = None
        self.model = None


class ElasticPropagator:
    """Velocity-stress time loop (elastic.py + rnn.py) over the native kernels."""

    def __init__(self, nz, nx, dt, h, bwidth=50, multiple=False, device=None):
        self.nz, self.nx = int(nz), int(nx)
        self.pitch = pitch_of(nx)
        self.dt, self.h = float(dt), float(h)
        self.bwidth = int(bwidth)
        self.multiple = bool(multiple)
        self.device = torch.device(device) if device is not None else torch.device("cuda")

    def grid(self, nshots):
        return grid_struct(self.nz, self.nx, self.pitch, nshots, self.dt, self.h)

    def model(self, vp, vs, rho, damp):
        """Pitched model planes and the six coefficient planes."""
        require_cuda(vp, "ElasticPropagator.model")
        check_cfl(vp, N.SCHEME_ELASTIC, 2, self.dt, self.h)
        planes = [to_pitched(m.detach().to(vp.device), self.pitch).contiguous() for m in (vp, vs, rho, damp)]
        coef = torch.empty(6, self.nz, self.pitch, dtype=torch.float32, device=vp.device)
        g = self.grid(1)
        N.call("sgb_elastic_coefficients", ctypes.byref(g), *[N.ptr(p) for p in planes], N.ptr(coef),
               N.stream_handle())
        m = N.ElasticModel(int(self.multiple), N.ptr(coef))
        return m, (planes, coef)

    def _pitched_fields(self, fields):
        return [to_pitched(f, self.pitch).contiguous() for f in fields]

    # -- one step (equation-module drop-in)
    def step(self, vp, vs, rho, damp, fields):
        m, keep = self.model(vp, vs, rho, damp)
        inp = self._pitched_fields(fields)
        out = [torch.empty_like(inp[0]) for _ in range(5)]
        g = self.grid(inp[0].shape[0])
        N.call("sgb_elastic_step", ctypes.byref(g), ctypes.byref(m), N.PTR5(*[t.data_ptr() for t in inp]),
               N.PTR5(*[t.data_ptr() for t in out]), N.stream_handle())
        return tuple(unpitched(o, self.nx) for o in out)

    def step_vjp(self, vp, vs, rho, damp, fields_in, stresses_out, grads_out):
        """(dJ/d inputs[5], dJ/dvp, dJ/dvs, dJ/drho) of one step."""
        m, (planes, coef) = self.model(vp, vs, rho, damp)
        vin = self._pitched_fields(fields_in[:2])
        sout = self._pitched_fields(stresses_out)
        gout = self._pitched_fields(grads_out)
        B = vin[0].shape[0]
        gin = [torch.empty_like(vin[0]) for _ in range(5)]
        gshot = [torch.zeros_like(vin[0]) for _ in range(3)]
        gmod = [torch.empty(self.nz, self.pitch, dtype=torch.float32, device=vin[0].device) for _ in range(3)]
        g = self.grid(B)
        s = N.stream_handle()
        N.call("sgb_elastic_step_vjp", ctypes.byref(g), ctypes.byref(m), N.PTR2(*[t.data_ptr() for t in vin]),
               N.PTR3(*[t.data_ptr() for t in sout]), N.PTR5(*[t.data_ptr() for t in gout]),
               N.PTR5(*[t.data_ptr() for t in gin]), N.PTR3(*[t.data_ptr() for t in gshot]), s)
        N.call("sgb_elastic_gradient", ctypes.byref(g), ctypes.byref(m), N.PTR3(*[t.data_ptr() for t in gshot]),
               N.ptr(planes[0]), N.ptr(planes[1]), N.ptr(planes[2]), None, 0,
               N.PTR3(*[t.data_ptr() for t in gmod]), s)
        return tuple(t[..., :self.nx] for t in gin), tuple(t[:, :self.nx] for t in gmod)

    # -- whole loop
    def forward(self, vp, vs, rho, damp, acq, io, nch, *, save_for_adjoint=False, illumination=False,
                ckpt_every=0):
        require_cuda(vp, "ElasticPropagator.forward")
        m, keep = self.model(vp, vs, rho, damp)
        B = acq.nshots
        dev = vp.device
        shape = (B, self.nz, self.pitch)
        buf = [torch.zeros(shape, dtype=torch.float32, device=dev) for _ in range(10)]
        records = torch.empty(acq.nt, max(acq.nrec, 1), nch, dtype=torch.float32, device=dev)
        illum = torch.zeros(self.nz, self.pitch, dtype=torch.float32, device=dev) if illumination else None
        state = ElasticState()
        bs = None
        if save_for_adjoint:
            iz0, iz1, ix0, ix1 = interior_box(self.nz, self.nx, self.bwidth, self.multiple)
            if iz1 <= iz0 or ix1 <= ix0:
                raise ValueError("grid too small for its boundary width")
            dpl = keep[0][3][:, :self.nx]
            if torch.count_nonzero(dpl[iz0:iz1, ix0:ix1]).item() != 0:
                raise ValueError("the damping profile is not zero inside the interior box; "
                                 "boundary-saving reconstruction needs an undamped interior")
            size = ctypes.c_int32(0)
            g1 = self.grid(B)
            N.call("sgb_ring_size", ctypes.byref(g1), iz0, iz1, ix0, ix1, 1, ctypes.byref(size))
            state.ring_store = torch.empty(acq.nt, 5, B, max(size.value, 1), dtype=torch.float32, device=dev)
            K = int(ckpt_every) if ckpt_every else 0
            nslots = acq.nt // K if K > 0 else 0
            state.ckpt_store = (torch.empty(max(nslots, 1), 5, *shape, dtype=torch.float32, device=dev)
                                if K > 0 else None)
            bs = N.BsStore(iz0, iz1, ix0, ix1, 1, size.value, N.ptr(state.ring_store), K,
                           N.ptr(state.ckpt_store))
            state.bs = bs
        cur = ctypes.c_int32(0)
        g = self.grid(B)
        q = acq.struct(records if acq.nrec else None, nch)
        N.call("sgb_elastic_forward", ctypes.byref(g), ctypes.byref(m), ctypes.byref(q), ctypes.byref(io),
               N.PTR10(*[b.data_ptr() for b in buf]), N.ptr(illum),
               ctypes.byref(bs) if bs is not None else None, ctypes.byref(cur), N.stream_handle())
        state.buf, state.cur, state.keep, state.model = buf, cur.value, keep, m
        return records[:, :acq.nrec], state, (illum[:, :self.nx] if illum is not None else None)

    def final_fields(self, state):
        return tuple(state.buf[5 * state.cur + f][..., :self.nx] for f in range(5))

    def backward(self, state, acq, io, nch, grad_records):
        """(dJ/dvp, dJ/dvs, dJ/drho), each (nz, nx), from dJ/d(records)."""
        B = acq.nshots
        dev = state.buf[0].device
        resid = torch.zeros(acq.nt, max(acq.nrec, 1), nch, dtype=torch.float32, device=dev)
        if acq.nrec:
            resid[:, :acq.nrec] = grad_records.to(torch.float32).reshape(acq.nt, acq.nrec, nch)
        shape = (B, self.nz, self.pitch)
        abuf = [torch.empty(shape, dtype=torch.float32, device=dev) for _ in range(10)]
        gshot = [torch.empty(shape, dtype=torch.float32, device=dev) for _ in range(3)]
        gmod = [torch.empty(self.nz, self.pitch, dtype=torch.float32, device=dev) for _ in range(3)]
        planes = state.keep[0]
        g = self.grid(B)
        q = acq.struct(resid, nch)
        N.call("sgb_elastic_backward", ctypes.byref(g), ctypes.byref(state.model), ctypes.byref(q),
               ctypes.byref(io), ctypes.byref(state.bs), N.PTR10(*[b.data_ptr() for b in state.buf]), state.cur,
               N.PTR10(*[b.data_ptr() for b in abuf]), N.PTR3(*[t.data_ptr() for t in gshot]),
               N.ptr(planes[0]), N.ptr(planes[1]), N.ptr(planes[2]), N.PTR3(*[t.data_ptr() for t in gmod]),
               N.stream_handle())
        return tuple(t[:, :self.nx] for t in gmod)


class _ElasticLoop(torch.autograd.Function):
    """Whole elastic loop as one differentiable op: (vp, vs, rho) -> records."""

    @staticmethod
    def forward(ctx, vp, vs, rho, prop, damp, acq, io, nch, illumination, ckpt_every):
        need = any(ctx.needs_input_grad[:3])
        rec, state, illum = prop.forward(vp, vs, rho, damp, acq, io, nch, save_for_adjoint=need,
                                         illumination=illumination, ckpt_every=ckpt_every)
        ctx.prop, ctx.acq, ctx.io, ctx.nch, ctx.state = prop, acq, io, nch, state
        if illum is not None:
            ctx.mark_non_differentiable(illum)
        return rec, illum if illum is not None else rec.new_zeros(0)

    @staticmethod
    def backward(ctx, grad_rec, grad_illum):
        if ctx.state.bs is None:
            return (None,) * 10
        gvp, gvs, grho = ctx.prop.backward(ctx.state, ctx.acq, ctx.io, ctx.nch, grad_rec.contiguous())
        ctx.state = None
        need = ctx.needs_input_grad
        return (gvp if need[0] else None, gvs if need[1] else None, grho if need[2] else None,
                None, None, None, None, None, None, None)


def elastic_records(vp, vs, rho, prop, damp, acq, io, nch, illumination=False, ckpt_every=0):
    """records (nt, nrec, nch) [, illum] of the elastic loop; differentiable in vp, vs, rho."""
    rec, illum = _ElasticLoop.apply(vp, vs, rho, prop, damp, acq, io, nch, illumination, ckpt_every)
    return rec, (illum if illumination else None)


def elastic_loop(models, geom, d, acq, source_illumination=False):
    """Whole loop for ``WaveRNN.forward`` (rnn.py:178-212) with the elastic
    equation: returns (records (nt, nrec, nch), illumination or None, None)."""
    from .engine import default_ckpt_every
    vp, vs, rho = [m.to(torch.float32) for m in models[:3]]
    nz, nx = vp.shape
    prop = ElasticPropagator(nz, nx, geom.dt, float(geom.h), geom.bwidth, geom.multiple, vp.device)
    io, nch = make_io(geom.source_type, geom.receiver_type)
    ck = geom.ckpt_every or default_ckpt_every(acq.nt)
    rec, illum = elastic_records(vp, vs, rho, prop, d.to(vp.device), acq, io, nch, source_illumination, ck)
    return rec, illum, None
