"""Born modelling for acoustic least-squares RTM
(seistorch/equations2d/acoustic_lsrtm_habc.py): a background field (h1, h2)
and a scattered field (sh1, sh2) driven by m vp^2 dt^2 lap(h1), both
blended by the hybrid absorbing boundary.  ``_time_step`` is one native
step of both fields (``sgb_born_step``) with its native VJP
(``sgb_habc_step_vjp`` per field); the whole loop with its dJ/dm adjoint
runs through ``WaveRNN`` (``engine.born_loop``)."""
import torch

from .. import engine
from ._acoustic_common import _scalar

spatial_order = 2
_CACHE = {}


def _propagator(shape, dt, h, multiple, device):
    key = (tuple(shape), dt, h, spatial_order, multiple, str(device))
    prop = _CACHE.get(key)
    if prop is None:
        prop = engine.BornPropagator(shape[-2], shape[-1], dt, h, spatial_order, 50, multiple, device)
        _CACHE[key] = prop
    return prop


class _BornStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vp, m, h1, h2, sh1, sh2, damp, prop, blend):
        ctx.prop, ctx.blend = prop, blend
        ctx.save_for_backward(vp, m, h1, h2, sh1, sh2, damp)
        return prop.step_born(vp, m, damp, h1, h2, sh1, sh2, blend)

    @staticmethod
    def backward(ctx, gp, gs):
        vp, m, h1, h2, sh1, sh2, damp = ctx.saved_tensors
        zero = lambda t: torch.zeros(h1.shape, dtype=torch.float32, device=h1.device) if t is None else t
        g = ctx.prop.step_vjp_born(vp, m, damp, h1, h2, sh1, sh2, zero(gp).contiguous(), zero(gs).contiguous(),
                                   ctx.blend)
        gh1, gh2, gsh1, gsh2, gvp, gm = g
        return (gvp.to(vp.dtype), gm.to(m.dtype), gh1.to(h1.dtype), gh2.to(h2.dtype), gsh1.to(sh1.dtype),
                gsh2.to(sh2.dtype), None, None, None)


def _step(args, multiple, blend=True):
    vp, m = args[0:2]
    h1, h2, sh1, sh2 = args[2:6]
    dt, h, b = args[6:9]
    engine.require_cuda(h1, "_time_step")
    squeeze = h1.ndim == 2
    if squeeze:
        h1, h2, sh1, sh2 = h1[None], h2[None], sh1[None], sh2[None]
    prop = _propagator(h1.shape, _scalar(dt), _scalar(h), multiple, h1.device)
    p0, s0 = _BornStep.apply(vp, m, h1, h2, sh1, sh2, b.to(h1.device), prop, blend)
    p0, s0 = p0.to(h1.dtype), s0.to(h1.dtype)
    if squeeze:
        return p0[0], h1[0], s0[0], sh1[0]
    return p0, h1, s0, sh1


def _time_step(*args, **kwargs):
    habcs = kwargs.get("habcs")
    multiple = habcs is not None and habcs[0] is None
    return _step(args, multiple)


def _backward(args, multiple):
    """Reverse step of the reference's boundary-saving path
    (acoustic_lsrtm_habc.py:33-86): the interior update of both fields
    without the one-way blend with (h1, h2) = (u_{n+1}, u_n), their saved
    strips restored, the source re-added to the background field."""
    from .utils import restore_boundaries
    h_bd, _, sh_bd, _ = args[-2]
    src_type, src_func, src_values = args[-1]
    p0, h1, s0, sh1 = _step(args[:9], multiple, blend=False)
    # tracked by autograd, as acoustic_lsrtm_habc.py:54-55 (no no_grad there)
    p0 = restore_boundaries(p0, h_bd, multiple=multiple)
    s0 = restore_boundaries(s0, sh_bd, multiple=multiple)
    p0 = src_func(p0, src_values, 1)
    return p0, h1, s0, sh1


def _time_step_backward(*args, **kwargs):
    return _backward(args, False)


def _time_step_backward_multiple(*args, **kwargs):
    return _backward(args, True)
