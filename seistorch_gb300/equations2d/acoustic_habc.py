"""Acoustic equation with the hybrid absorbing boundary
(seistorch/equations2d/acoustic_habc.py): undamped interior update followed by
the one-way-wave blend on the four 50-cell strips, fused in one kernel.
``d`` is the HABC blend weight (habc.generate_habc_coefficients_2d)."""
from . import _acoustic_common as _c

spatial_order = 2


def _time_step(*args, **kwargs):
    habcs = kwargs.get("habcs")
    multiple = habcs is not None and habcs[0] is None
    return _c.time_step(args, spatial_order, "habc", multiple)


def _time_step_backward(*args, **kwargs):
    return _c.time_step_backward(args, spatial_order, "habc", False)


def _time_step_backward_multiple(*args, **kwargs):
    return _c.time_step_backward(args, spatial_order, "habc", True)
