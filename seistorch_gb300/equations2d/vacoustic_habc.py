"""Viscoacoustic equation with the hybrid absorbing boundary
(seistorch/equations2d/vacoustic_habc.py): 2 h1 - h2 + vp^2 dt^2 lap(h1) with
the phase correction -(1 - sqrt(Q^2 + 1)) Q^-2 vp^2 dt^2 lap(h1) and the
amplitude term -(dt t vp / 2) K(h1 - h2), K = real(ifft2(|k| fft2(.))), then
the one-way-wave blend (``engine.vacoustic_coefficients`` for kv and the
damping plane; omega = 16.5 in the forward step, 5.0 in the reverse steps, as
the reference).  ``_time_step`` is one native step (``sgb_vacoustic_step``:
the batched 2-D FFT term and the HABC step kernel) with its native VJP; the
reverse steps are the unblended update with the strips restored under
autograd and the source re-added (vacoustic_habc.py:117-206)."""
from .. import engine
from ._acoustic_common import _scalar

spatial_order = 2
_CACHE = {}


def _propagator(shape, dt, h, multiple, device):
    key = (tuple(shape), dt, h, spatial_order, multiple, str(device))
    prop = _CACHE.get(key)
    if prop is None:
        prop = engine.VacousticPropagator(shape[-2], shape[-1], dt, h, spatial_order, 50, multiple, device)
        _CACHE[key] = prop
    return prop


def _step(args, multiple, blend=True, omega=16.5):
    vp, Q = args[0:2]
    h1, h2 = args[2:4]
    dt, h, b = args[4:7]
    engine.require_cuda(h1, "_time_step")
    squeeze = h1.ndim == 2
    if squeeze:
        h1, h2 = h1[None], h2[None]
    prop = _propagator(h1.shape, _scalar(dt), _scalar(h), multiple, h1.device)
    y = engine.VacousticStep.apply(vp, Q, h1, h2, b.to(h1.device), prop, blend, omega).to(h1.dtype)
    return (y[0], h1[0]) if squeeze else (y, h1)


def _time_step(*args, **kwargs):
    habcs = kwargs.get("habcs")
    multiple = habcs is not None and habcs[0] is None
    return _step(args, multiple)


def _backward(args, multiple):
    from .utils import restore_boundaries
    h_bd, _ = args[-2]
    src_type, src_func, src_values = args[-1]
    y, h1 = _step(args[:7], multiple, blend=False, omega=5.0)
    # tracked by autograd, as vacoustic_habc.py:150,197 (no no_grad there)
    y = restore_boundaries(y, h_bd, multiple=multiple)
    y = src_func(y, src_values, 1)
    return y, h1


def _time_step_backward(*args, **kwargs):
    return _backward(args, False)


def _time_step_backward_multiple(*args, **kwargs):
    return _backward(args, True)
