"""Acquisition set-up (seistorch/setup.py:261-483, seistorch/coords.py:127-156,
seistorch/rnn.py:35-73): shift grid coordinates by the boundary width and
merge per-shot sources / receivers into one batched source and probe."""
import torch

from .probe import WaveIntensityProbe, WaveProbe
from .source import WaveSource


def setup_src_coords(coords, bwidth, multiple=False):
    """Source coordinates + boundary width; 2D top unshifted with multiple
    (setup.py:452-483)."""
    kwargs = {}
    for key, value in zip(["x", "y", "z"], coords):
        if value is not None and not isinstance(value, (int, float)):
            raise TypeError(f"The source location must be a number, got {type(value)}.")
        kwargs[key] = value + bwidth if isinstance(value, (int, float)) else value
    if "z" not in kwargs and multiple and bool(kwargs.get("y")):
        kwargs["y"] -= bwidth
    if "z" in kwargs:
        raise NotImplementedError("seistorch_gb300 implements the 2D path only")
    return WaveSource(**{k: int(v) for k, v in kwargs.items()})


def setup_rec_coords(coords, bwidth, multiple=False):
    """Receiver coordinates + boundary width (setup.py:386-415)."""
    kwargs = {}
    for key, value in zip(["x", "y", "z"], coords):
        kwargs[key] = [v + bwidth if v is not None else None for v in value]
    if "z" not in kwargs and multiple:
        kwargs["y"] = [v - bwidth if v is not None else None for v in kwargs["y"]]
    if "z" in kwargs:
        raise NotImplementedError("seistorch_gb300 implements the 2D path only")
    kwargs = {k: [int(v) for v in vals] for k, vals in kwargs.items()}
    return [WaveIntensityProbe(**kwargs)]


def setup_acquisition(shots, src_list, rec_list, cfg, *args, **kwargs):
    bwidth = cfg["geom"]["boundary"]["width"]
    multiple = cfg["geom"]["multiple"]
    sources, receivers = [], []
    for shot in shots:
        sources.append(setup_src_coords(src_list[shot], bwidth, multiple))
        receivers.extend(setup_rec_coords(rec_list[shot], bwidth, multiple))
    return sources, receivers


def merge_sources_with_same_keys(sources):
    super_source = {}
    batchindices = []
    for bidx, source in enumerate(sources):
        for key, val in source.coords().items():
            super_source.setdefault(key, []).append(val)
        batchindices.append(bidx * torch.ones(1, dtype=torch.int64))
    super_source = {k: torch.cat([v.reshape(-1) for v in vals]) for k, vals in super_source.items()}
    return batchindices, super_source


def merge_receivers_with_same_keys(probes):
    super_probes = {}
    batchindices = []
    reccounts = []
    for bidx, probe in enumerate(probes):
        coords = probe.coords()
        n = 0
        for key, val in coords.items():
            super_probes.setdefault(key, []).append(val.reshape(-1))
            n = val.numel()
        reccounts.append(n)
        batchindices.append(bidx * torch.ones(n, dtype=torch.int64))
    for key in super_probes:
        super_probes[key] = torch.cat(super_probes[key], dim=0)
    return reccounts, torch.cat(batchindices), super_probes


def single2batch(src, rec, cfg, dev):
    """Batched source / probe from per-shot coordinate tensors
    (coords.py:127-156): src = [x (nshots,), y (nshots,)],
    rec = (ncoords, nrec, nshots)."""
    rec = rec.permute(2, 0, 1).cpu().numpy().tolist()
    src = torch.stack(src).cpu().numpy().T.tolist()
    shots = list(range(len(src)))
    padded_src, padded_rec = setup_acquisition(shots, src, rec, cfg)
    bidx_source, sourcekeys = merge_sources_with_same_keys(padded_src)
    super_source = WaveSource(bidx_source, **sourcekeys).to(dev)
    reccounts, bidx_receivers, reckeys = merge_receivers_with_same_keys(padded_rec)
    super_probes = WaveProbe(bidx_receivers, **reckeys).to(dev)
    super_probes.reccounts = reccounts
    return super_source, super_probes
