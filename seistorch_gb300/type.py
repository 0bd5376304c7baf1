"""Record container (seistorch/type.py:7-97)."""
import torch


class TensorList(list):
    """A list of per-shot record tensors (nt, nrec, nch)."""

    def __init__(self, input_list=()):
        super().__init__()
        self.data = [t if isinstance(t, torch.Tensor) else torch.as_tensor(t) for t in input_list]

    @property
    def device(self):
        return self.data[0].device

    @property
    def shape(self):
        return (len(self.data),)

    def append(self, item):
        self.data.append(item if isinstance(item, torch.Tensor) else torch.as_tensor(item))

    def extend(self, items):
        for it in items:
            self.append(it)

    def cuda(self):
        self.data = [t.cuda() for t in self.data]
        return self

    def has_nan(self):
        """Raise ValueError on NaN (type.py:41-46, called at rnn.py:215)."""
        for t in self.data:
            if isinstance(t, torch.Tensor) and torch.isnan(t).any():
                raise ValueError("The tensor list contains NaN values.")
        return False

    def numpy(self):
        self.data = [t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else t for t in self.data]
        return self

    def stack(self):
        """Zero-pad to the largest (nt, nrec) and stack (type.py:54-57)."""
        max_shape = max(t.shape for t in self.data)
        padded = [torch.nn.functional.pad(t, (0, 0, 0, max_shape[1] - t.shape[1], 0, max_shape[0] - t.shape[0]))
                  if t.ndim == 3 else
                  torch.nn.functional.pad(t, (0, max_shape[1] - t.shape[1], 0, max_shape[0] - t.shape[0]))
                  for t in self.data]
        return torch.stack(padded, dim=0)

    def tensor(self):
        return self.data

    def to(self, device):
        self.data = [t.to(device) for t in self.data]
        return self

    def tolist(self):
        return self

    def __getitem__(self, index):
        return self.data[index]

    def __iter__(self):
        return iter(self.data)

    def __len__(self):
        return len(self.data)

    def __str__(self):
        return str(self.data)
