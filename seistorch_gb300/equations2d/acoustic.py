"""2nd-order acoustic equation with PML (seistorch/equations2d/acoustic.py).

``_time_step(vp, h1, h2, dt, h, d, habcs=None) -> (y, h1)`` runs one native
step; autograd flows to vp, h1 and h2 through the native single-step VJP.
``spatial_order`` is the module-level order (2 by default, as the reference
hard-wires at acoustic.py:55); set it to 4, 6 or 8 for higher orders.
"""
from . import _acoustic_common as _c

spatial_order = 2


def _time_step(*args, **kwargs):
    return _c.time_step(args, spatial_order, "pml")


def _time_step_backward(*args, **kwargs):
    return _c.time_step_backward(args, spatial_order, "pml", False)


def _time_step_backward_multiple(*args, **kwargs):
    return _c.time_step_backward(args, spatial_order, "pml", True)
