"""Autotuner of the acoustic tile-pipeline variants.

The forward and adjoint PML kernels are compiled in a few variants (rows per
tile, warps per CTA, pipeline stages, whether the previous field travels
through the TMA stage).  Which one is fastest depends on the grid: the
number of tiles against the 152 SMs, the share of halo rows, L2 reuse of
the coefficient planes.  ``tune_grid`` times every variant on a short
synthetic run of the given shape (CUDA events on the current stream, after
a warm-up) and caches the winner per (nz, nx, shots, order); ``select``
makes a winner current for the process (``sgb_set_stream_config``).  An
uneven batch of several grids runs in one persistent launch and therefore
one variant: ``tune_batch`` times the per-grid winners on the batch itself.
"""
import ctypes
import json
import os

import torch

from . import _native as N

FWD_VARIANTS = [  # (rows per tile, warps, stages, previous field via TMA)
    (16, 4, 3, False), (16, 4, 3, True), (8, 4, 4, True), (32, 8, 2, True), (16, 4, 2, True), (8, 4, 3, True)]
BWD_VARIANTS = [  # (rows per tile, warps, stages, point rows via TMA: 0 none, 1 U_j and nu_{j+2}, 2 also g, k)
    (8, 4, 2, 0), (8, 2, 2, 0), (16, 4, 2, 0), (8, 4, 3, 0), (8, 4, 2, 1), (8, 4, 2, 2)]
DEFAULT = (4, 4)

_CACHE = {}


def select(fwd_cfg, bwd_cfg):
    """Make (fwd_cfg, bwd_cfg) the variants of later PML calls in this process."""
    N.call("sgb_set_stream_config", int(fwd_cfg), int(bwd_cfg), 0)


def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _setup(nz, nx, nshots, order, dt, h, bwidth, device, steps):
    from . import engine
    from .pml import generate_pml_coefficients_2d
    from .utils import ricker_wave
    prop = engine.AcousticPropagator(nz, nx, dt, h, order, "pml", bwidth, False, device)
    vp = torch.full((nz, nx), 2500.0, dtype=torch.float32, device=device)
    d = generate_pml_coefficients_2d((nz, nx), bwidth).to(device=device, dtype=torch.float32)
    xs = torch.linspace(bwidth, nx - bwidth - 1, nshots).round().int().tolist()
    src = [[(bwidth + 2, int(x))] for x in xs]
    rec = [([bwidth + 2] * (nx - 2 * bwidth), list(range(bwidth, nx - bwidth)))] * nshots
    wav = ricker_wave(10.0, dt, steps, delay=20, dtype="numpy")
    acq = engine.Acquisition(nz, nx, src, rec, wav, device)
    return prop, vp, d, acq


def tune_grid(nz, nx, nshots, order, dt=0.001, h=10.0, bwidth=50, device=None, steps=24, adjoint=True,
              repeats=2):
    """Fastest (fwd_cfg, bwd_cfg) for one grid; returns (best, timings_ms)."""
    key = (int(nz), int(nx), int(nshots), int(order), bool(adjoint))
    if key in _CACHE:
        return _CACHE[key]
    device = torch.device(device or "cuda")
    prop, vp, d, acq = _setup(nz, nx, nshots, order, dt, h, bwidth, device, steps)
    times = {"fwd": {}, "bwd": {}}
    for fi in range(len(FWD_VARIANTS)):
        select(fi, DEFAULT[1])
        prop.forward(vp, d, acq)  # warm-up (module load, first-launch attribute setup)
        best = float("inf")
        for _ in range(repeats):
            a, b = _events()
            a.record()
            prop.forward(vp, d, acq)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        times["fwd"][fi] = best
    fbest = min(times["fwd"], key=times["fwd"].get)
    bbest = DEFAULT[1]
    if adjoint:
        select(fbest, DEFAULT[1])
        ck = max(4, steps // 4)
        rec, state, _ = prop.forward(vp, d, acq, save_for_adjoint=True, ckpt_every=ck)
        resid = rec.contiguous()
        for bi in range(len(BWD_VARIANTS)):
            select(fbest, bi)
            prop.backward(state, acq, resid)
            best = float("inf")
            for _ in range(repeats):
                rec, state, _ = prop.forward(vp, d, acq, save_for_adjoint=True, ckpt_every=ck)
                a, b = _events()
                a.record()
                prop.backward(state, acq, resid)
                b.record()
                torch.cuda.synchronize()
                best = min(best, a.elapsed_time(b))
            times["bwd"][bi] = best
        bbest = min(times["bwd"], key=times["bwd"].get)
    out = ((fbest, bbest), times)
    _CACHE[key] = out
    select(fbest, bbest)
    return out


def tune_batch(run, candidates, repeats=2):
    """Time ``run()`` (one uneven-batch forward) under each candidate forward
    variant and keep the fastest; returns (best_fwd_cfg, timings_ms)."""
    times = {}
    for fi in sorted(set(int(c) for c in candidates)):
        select(fi, DEFAULT[1])
        run()
        best = float("inf")
        for _ in range(repeats):
            a, b = _events()
            a.record()
            run()
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        times[fi] = best
    fbest = min(times, key=times.get)
    select(fbest, DEFAULT[1])
    return fbest, times


def save(path):
    """Write the cached winners to a JSON file."""
    with open(path, "w") as f:
        json.dump([{"key": list(k), "fwd": v[0][0], "bwd": v[0][1]} for k, v in _CACHE.items()], f)


def load(path):
    """Read winners written by ``save`` into the cache (timings are not kept)."""
    if not os.path.exists(path):
        return
    with open(path) as f:
        for e in json.load(f):
            k = e["key"]
            _CACHE[(int(k[0]), int(k[1]), int(k[2]), int(k[3]), bool(k[4]))] = ((e["fwd"], e["bwd"]), {})
