"""Time-step dispatch (seistorch/cell.py:9-77).

``WaveCell.forward`` keeps the reference's per-step contract (calls the
equation module's ``_time_step``); ``WaveRNN`` bypasses it and hands the whole
loop to the native engine in one call.
"""
import torch

from .habc import bound_mask


class WaveCell(torch.nn.Module):
    def __init__(self, geometry, forward_func=None, backward_func=None):
        super().__init__()
        self.geom = geometry
        self.register_buffer("dt", torch.tensor(float(self.geom.dt)))
        self.forward_func = forward_func
        self.backward_func = backward_func

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
        habcs = getattr(self, "habc_masks", None) if self.geom.use_habc else None
        geoms = self.dt, self.geom.h, self.geom.d
        return self.forward_func(*model_vars, *wavefields, *geoms, habcs=habcs)
