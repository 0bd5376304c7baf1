"""Time-step dispatch (seistorch/cell.py:9-77).

``WaveCell.forward`` keeps the reference's per-step contract: it calls the
equation module's ``_time_step`` (autograd through its native VJP when a
model parameter requires grad), or, with ``boundary_saving`` and
``inversion``, the boundary-saving step of ``checkpoint.py`` with the
module's ``_time_step_backward``.  ``WaveRNN`` bypasses the cell and hands
the whole loop to the native engine in one call.
"""
import inspect

import torch

from .checkpoint import ReverseState, boundary_saving_step
from .eqconfigure import Parameters
from .habc import bound_mask


class WaveCell(torch.nn.Module):
    def __init__(self, geometry, forward_func=None, backward_func=None):
        super().__init__()
        self.geom = geometry
        self.register_buffer("dt", torch.tensor(float(self.geom.dt)))
        self.forward_func = forward_func
        self.backward_func = backward_func
        # second-order equations use the acoustic protocol of the
        # boundary-saving reverse sweep (cell.py:22-28)
        mod = inspect.getmodule(forward_func) if forward_func is not None else None
        name = mod.__name__.split(".")[-1] if mod is not None else ""
        self.second_order = name in Parameters.secondorder_equations()
        self.reverse_state = ReverseState()

    def setup_habc(self, batchsize):
        if self.geom.use_habc:
            self.habc_masks = bound_mask(*self.geom.domain_shape, self.geom.bwidth, self.geom.h.device,
                                         batchsize, return_idx=True, multiple=self.geom.multiple)

    def parameters(self, recurse=True):
        for p in self.geom.parameters():
            yield p

    def get_parameters(self, key=None, recursive=True, implicit=False):
        yield getattr(self.geom, key)

    def forward(self, wavefields, model_vars, **kwargs):
        """One step (cell.py:50-77).  Keywords: ``is_last_frame`` and
        ``source`` ([source types, source module, source values]), used by
        the boundary-saving inversion."""
        habcs = getattr(self, "habc_masks", None) if self.geom.use_habc else None
        geoms = self.dt, self.geom.h, self.geom.d
        if getattr(self.geom, "boundary_saving", False) and getattr(self.geom, "inversion", False):
            return boundary_saving_step(self.reverse_state, self.forward_func, self.backward_func,
                                        kwargs.get("source"), bool(kwargs.get("is_last_frame", False)),
                                        len(model_vars), self.second_order, *model_vars, *wavefields, *geoms,
                                        habcs=habcs)
        return self.forward_func(*model_vars, *wavefields, *geoms, habcs=habcs)
