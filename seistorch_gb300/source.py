"""Source module (seistorch/source.py:6-57).

In the reference ``forward2d`` adds ``smask * X`` to the field every step;
here the whole loop runs in the CUDA step kernel, which injects at the
source points directly.  ``forward2d`` stays available for per-step loops.
"""
import torch


def _as_index(value):
    if value is None:
        return None
    return torch.as_tensor(value, dtype=torch.int64).reshape(-1) if not isinstance(value, torch.Tensor) \
        else value.to(torch.int64).reshape(-1)


class WaveSource(torch.nn.Module):
    def __init__(self, bidx=None, second_order_equation=False, **kwargs):
        super().__init__()
        self._ndim = len(kwargs)
        self.coord_labels = list(kwargs.keys())
        for key, value in kwargs.items():
            self.register_buffer(key, _as_index(value))
        self.bidx = bidx
        self._source_encoding = False
        self.second_order_equation = second_order_equation
        self.smask = None

    @property
    def ndim(self):
        return self._ndim

    @property
    def source_encoding(self):
        return self._source_encoding

    @source_encoding.setter
    def source_encoding(self, value):
        self._source_encoding = value

    def coords(self):
        return dict(zip(self.coord_labels, [getattr(self, k) for k in self.coord_labels]))

    def forward(self, Y, X, dt=1.0):
        return self.forward2d(Y, X, dt)

    def forward2d(self, Y, X, dt=1.0):
        """Y += smask * X (clone first for 2nd-order equations); with source
        encoding Y[..., y, x] += dt * X (source.py:47-57)."""
        Y_new = Y.clone() if self.second_order_equation else Y
        if not self.source_encoding:
            if self.smask is None:
                smask = torch.zeros_like(Y)
                for idx in range(self.x.size(0)):
                    smask[idx, self.y[idx], self.x[idx]] = 1.0
                self.smask = smask
            Y_new += self.smask * X
        else:
            Y_new[..., self.y, self.x] += dt * X
        return Y_new
