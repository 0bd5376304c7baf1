"""VTI acoustic equation with the hybrid absorbing boundary
(seistorch/equations2d/vti_habc2.py): 2 p1 - p2 + vp^2 dt^2 ((1 + 2 eps) + sk)
lap_x(p1) + vp^2 dt^2 (1 + sk) lap_z(p1), then the one-way-wave blend, with
the reference's per-cell sk of eps, delta and the FFT frequencies
(``engine.vti_coefficients``).  ``_time_step`` is one native step
(``sgb_vti_step``) with its native VJP (``sgb_habc_step_vjp``) for autograd;
the whole loop with its adjoint runs through ``WaveRNN``
(``engine.vti_loop``)."""
import torch

from .. import engine
from ._acoustic_common import _scalar

_CACHE = {}


def _propagator(shape, dt, h, multiple, device):
    key = (tuple(shape), dt, h, multiple, str(device))
    prop = _CACHE.get(key)
    if prop is None:
        prop = engine.VTIPropagator(shape[-2], shape[-1], dt, h, 50, multiple, device)
        _CACHE[key] = prop
    return prop


class _VTIStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vp, eps, delta, p1, p2, damp, prop, blend):
        ctx.prop, ctx.blend = prop, blend
        ctx.save_for_backward(vp, eps, delta, p1, p2, damp)
        return prop.step_vti(vp, eps, delta, damp, p1, p2, blend)

    @staticmethod
    def backward(ctx, gy):
        vp, eps, delta, p1, p2, damp = ctx.saved_tensors
        gu, gum, gm = ctx.prop.step_vjp_vti(vp, eps, delta, damp, p1, p2, gy.contiguous(), ctx.blend)
        return (gm[0].to(vp.dtype), gm[1].to(eps.dtype), gm[2].to(delta.dtype), gu.to(p1.dtype), gum.to(p2.dtype),
                None, None, None)


def _step(args, multiple, blend=True):
    vp, eps, delta = args[0:3]
    p1, p2 = args[3:5]
    dt, h, b = args[5:8]
    engine.require_cuda(p1, "_time_step")
    squeeze = p1.ndim == 2
    if squeeze:
        p1, p2 = p1[None], p2[None]
    prop = _propagator(p1.shape, _scalar(dt), _scalar(h), multiple, p1.device)
    y = _VTIStep.apply(vp, eps, delta, p1, p2, b.to(p1.device), prop, blend).to(p1.dtype)
    return (y[0], p1[0]) if squeeze else (y, p1)


def _time_step(*args, **kwargs):
    habcs = kwargs.get("habcs")
    multiple = habcs is not None and habcs[0] is None
    return _step(args, multiple)


def _backward(args, multiple):
    """Reverse step of the reference's boundary-saving path
    (vti_habc2.py:62-146): the interior update without the one-way blend
    with (p1, p2) = (u_{n+1}, u_n), saved strips restored, the source
    re-added."""
    from .utils import restore_boundaries
    h_bd, _ = args[-2]
    src_type, src_func, src_values = args[-1]
    y, p1 = _step(args[:8], multiple, blend=False)
    # tracked by autograd, as vti_habc2.py:99 (no no_grad there): the
    # restored cells take their values, and their gradients, from the strips
    y = restore_boundaries(y, h_bd, multiple=multiple)
    y = src_func(y, src_values, 1)
    return y, p1


def _time_step_backward(*args, **kwargs):
    return _backward(args, False)


def _time_step_backward_multiple(*args, **kwargs):
    return _backward(args, True)
