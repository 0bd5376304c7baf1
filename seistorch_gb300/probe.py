"""Receiver modules (seistorch/probe.py:6-56): nearest-grid sampling
``x[bidx, y, x]``.  The CUDA step kernel gathers the receivers itself; the
modules carry the coordinates and the per-shot counts."""
import torch


class WaveProbe(torch.nn.Module):
    def __init__(self, batchidx=None, reccounts=(), **kwargs):
        super().__init__()
        self._ndim = len(kwargs)
        self.coord_labels = list(kwargs.keys())
        for key, value in kwargs.items():
            self.register_buffer(key, torch.as_tensor(value, dtype=torch.int64))
        self.batchsize = self.x.size(0) if self.x.ndim > 1 else 1
        self.bidx = batchidx
        self.reccounts = list(reccounts)

    @property
    def ndim(self):
        return self._ndim

    def coords(self):
        return dict(zip(self.coord_labels, [getattr(self, k) for k in self.coord_labels]))

    def forward(self, x):
        return self.forward2d(x)

    def forward2d(self, x):
        return x[self.bidx, self.y, self.x]


class WaveIntensityProbe(WaveProbe):
    def __init__(self, **kwargs):
        super().__init__(**kwargs)
