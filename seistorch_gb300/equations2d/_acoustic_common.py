"""Per-step acoustic op shared by acoustic.py and acoustic_habc.py."""
import torch

from .. import engine

_CACHE = {}


def _scalar(v):
    return float(v.item()) if isinstance(v, torch.Tensor) else float(v)


def propagator(shape, dt, h, order, boundary, multiple, device):
    key = (tuple(shape), dt, h, order, boundary, multiple, str(device))
    prop = _CACHE.get(key)
    if prop is None:
        prop = engine.AcousticPropagator(shape[-2], shape[-1], dt, h, order, boundary, 50, multiple, device)
        _CACHE[key] = prop
    return prop


class _AcousticStep(torch.autograd.Function):
    """One native step y = step(vp, h1, h2) with its native VJP: the PML
    step (sgb_acoustic_step_vjp) or the HABC step, blended or not
    (sgb_habc_step_vjp)."""

    @staticmethod
    def forward(ctx, vp, h1, h2, damp, prop, blend):
        ctx.prop, ctx.blend = prop, blend
        ctx.save_for_backward(vp, h1, h2, damp)
        return prop.step(vp, damp, h1.to(torch.float32), h2.to(torch.float32), blend)

    @staticmethod
    def backward(ctx, gy):
        vp, h1, h2, damp = ctx.saved_tensors
        gy = gy.contiguous().to(torch.float32)
        if ctx.prop.boundary == engine.BOUNDARY_PML:
            gu, gum, gvp = ctx.prop.step_vjp(vp, damp, h1.to(torch.float32), gy, None)
        else:
            gu, gum, gvp = ctx.prop.step_vjp_habc(vp, damp, h1, h2, gy, ctx.blend)
        return gvp.to(vp.dtype), gu.to(h1.dtype), gum.to(h2.dtype), None, None, None


def time_step(args, order, boundary, multiple=False, blend=True):
    c = args[0]
    h1, h2 = args[1:3]
    dt, h, b = args[3:6]
    engine.require_cuda(h1, "_time_step")
    if h1.ndim == 2:
        h1, h2 = h1[None], h2[None]
    prop = propagator(h1.shape, _scalar(dt), _scalar(h), order, boundary, multiple, h1.device)
    y = _AcousticStep.apply(c, h1, h2, b.to(h1.device), prop, blend)
    return y.to(h1.dtype), h1


def time_step_backward(args, order, boundary, multiple):
    """Reverse step of the reference's boundary-saving path with (h1, h2) =
    (u_{n+1}, u_n): for PML the forward formula with its damping
    (acoustic.py:88-137), for HABC the plain undamped update without the
    one-way blend (acoustic_habc.py:223-268); then the saved strips are
    restored and the source re-added.  Differentiable (the reference
    back-propagates through it, checkpoint_new.py:180-199)."""
    from .utils import restore_boundaries
    h_bd, _ = args[-2]
    src_type, src_func, src_values = args[-1]
    y, h1 = time_step(args[:6], order, boundary, multiple, blend=boundary != "habc")
    with torch.no_grad():
        y = restore_boundaries(y, h_bd, multiple=multiple)
    y = src_func(y, src_values, 1)
    return y, h1
