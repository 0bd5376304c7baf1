"""Isotropic elastic velocity-stress equation (seistorch/equations2d/elastic.py).

``_time_step(vp, vs, rho, vx, vz, txx, tzz, txz, dt, h, d) -> (vx, vz, txx,
tzz, txz)`` runs one native step (elastic.py:7-37); autograd flows to the
model and to the five input fields through the native single-step VJP.

``_time_step_backward(_multiple)`` is the reference's boundary-saving reverse
step (elastic.py:39-207): the -dt update evaluated on the sub-grid
[49:-49] (rows [0:-49] with ``multiple``), written back one cell further in,
velocities first and stresses from the reversed velocities, the saved strips
restored and the sources taken out (``src_func(..., -1)``).  It is kept with
the reference's semantics for callers that drive the per-step reverse
themselves; ``WaveRNN`` gradients use the fused native adjoint instead.
"""
import torch

from .. import elastic_engine
from .utils import diff_using_roll, restore_boundaries

NPML = 49
N = 1

_CACHE = {}


def _scalar(v):
    return float(v.item()) if isinstance(v, torch.Tensor) else float(v)


def _propagator(shape, dt, h, device):
    key = (tuple(shape), dt, h, str(device))
    prop = _CACHE.get(key)
    if prop is None:
        prop = elastic_engine.ElasticPropagator(shape[-2], shape[-1], dt, h, 50, False, device)
        _CACHE[key] = prop
    return prop


class _ElasticStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vp, vs, rho, vx, vz, txx, tzz, txz, damp, prop):
        ctx.prop = prop
        f32 = [t.to(torch.float32) for t in (vx, vz, txx, tzz, txz)]
        out = prop.step(vp, vs, rho, damp, f32)
        ctx.save_for_backward(vp, vs, rho, damp, f32[0], f32[1], out[2], out[3], out[4])
        return out

    @staticmethod
    def backward(ctx, *gouts):
        vp, vs, rho, damp, vx, vz, sxx, szz, sxz = ctx.saved_tensors
        gouts = [g if g is not None else torch.zeros_like(vx) for g in gouts]
        gin, (gvp, gvs, grho) = ctx.prop.step_vjp(vp, vs, rho, damp, (vx, vz), (sxx, szz, sxz),
                                                  [g.contiguous().to(torch.float32) for g in gouts])
        return (gvp.to(vp.dtype), gvs.to(vs.dtype), grho.to(rho.dtype), *gin, None, None)


def _time_step(*args, **kwargs):
    vp, vs, rho = args[0:3]
    fields = list(args[3:8])
    dt, h, d = args[8:11]
    squeeze = fields[0].ndim == 2
    if squeeze:
        fields = [f[None] for f in fields]
    prop = _propagator(fields[0].shape, _scalar(dt), _scalar(h), fields[0].device)
    out = _ElasticStep.apply(vp, vs, rho, *fields, d.to(fields[0].device), prop)
    out = tuple(o.to(args[3].dtype) for o in out)
    return tuple(o[0] for o in out) if squeeze else out


def _reverse(args, multiple):
    vp, vs, rho = (a.unsqueeze(0) for a in args[0:3])
    vx, vz, txx, tzz, txz = args[3:8]
    dt, h, d = args[8:11]
    d = d.unsqueeze(0)
    bds = args[-2]
    src_type, src_func, src_values = args[-1]
    top = 0 if multiple else NPML
    comp = (slice(None), slice(top, -NPML), slice(NPML, -NPML))          # evaluated on this sub-grid
    upd = (slice(None), slice(top if multiple else NPML + N, -NPML - N), slice(NPML + N, -NPML - N))
    inner = (slice(None), slice(0 if multiple else N, -N), slice(N, -N))  # its part written back
    lam = rho * (vp ** 2 - 2 * vs ** 2)
    mu = rho * vs ** 2
    c = 0.5 * dt * d[comp]
    inv = 1.0 / (1 + c)
    # velocities from the current stresses, run backwards in time
    dv_x = diff_using_roll(txx, 2, False)[comp] + diff_using_roll(txz, 1, False)[comp]
    dv_z = diff_using_roll(txz, 2)[comp] + diff_using_roll(tzz, 1)[comp]
    nvx, nvz = vx.clone(), vz.clone()
    nvx[upd] = (inv * (-dt / (rho[comp] * h) * dv_x + (1 - c) * vx[comp]))[inner]
    nvz[upd] = (inv * (-dt / (rho[comp] * h) * dv_z + (1 - c) * vz[comp]))[inner]
    nvx = restore_boundaries(nvx, bds[0], multiple=multiple)
    nvz = restore_boundaries(nvz, bds[1], multiple=multiple)
    # stresses from the reversed velocities (differences taken on the sub-grid)
    svx, svz = nvx[comp], nvz[comp]
    ax = diff_using_roll(svx, 2)
    bz = diff_using_roll(svz, 1, False)
    cz = diff_using_roll(svx, 1)
    cx = diff_using_roll(svz, 2, False)
    l, m = lam[comp], mu[comp]
    ntxx, ntzz, ntxz = txx.clone(), tzz.clone(), txz.clone()
    ntxx[upd] = (inv * (-dt / h * ((l + 2 * m) * ax + l * bz) + (1 - c) * txx[comp]))[inner]
    ntzz[upd] = (inv * (-dt / h * ((l + 2 * m) * bz + l * ax) + (1 - c) * tzz[comp]))[inner]
    ntxz[upd] = (inv * (-dt * m / h * (cx + cz) + (1 - c) * txz[comp]))[inner]
    ntxx = restore_boundaries(ntxx, bds[2], multiple=multiple)
    ntzz = restore_boundaries(ntzz, bds[3], multiple=multiple)
    ntxz = restore_boundaries(ntxz, bds[4], multiple=multiple)
    out = {"vx": nvx, "vz": nvz, "txx": ntxx, "tzz": ntzz, "txz": ntxz}
    for s in src_type:
        out[s].data.copy_(src_func(out[s], src_values, -1))
    return out["vx"], out["vz"], out["txx"], out["tzz"], out["txz"]


def _time_step_backward(*args, **kwargs):
    return _reverse(args, False)


def _time_step_backward_multiple(*args, **kwargs):
    return _reverse(args, True)
