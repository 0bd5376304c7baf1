"""Timed CPU baseline of the acoustic L2-gradient step (oracle port).

TEST AND CPU-BASELINE INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): used by
``bench.py`` as the CPU baseline and as its ``--impl reference`` arm.

The reference's own implementation is Python on PyTorch and is not shipped
with this package, so the baseline is this numpy restatement of the same
discrete algorithm (measured 13.7x faster than the reference's PyTorch CPU
path with pure autograd on the same sample and thread count) (forward loop of rnn.py:178-205 with the update of
acoustic.py:73-86, the L2 adjoint source of loss.py:409-421, and the exact
adjoint whose result the reference gets from autograd), in float32 like the
reference's default dtype.  One spawned process per shot runs a bounded
number of time steps; the rate is grid-point updates (forward + adjoint
counted once per point-step) per second of wall time.
"""
import multiprocessing as mp
import os
import time

import numpy as np


def _one_shot(args):
    vp, d, dt, h, wavelet, src, rec, order = args
    from oracle import adjoint, fd2d
    t0 = time.perf_counter()
    out = fd2d.forward("acoustic", {"vp": vp}, d, dt, h, wavelet, [src], [rec], order=order,
                       dtype=np.float32)
    syn = out["records"][0]
    resid = [2.0 * syn]  # L2 against zero data: the adjoint source is 2 syn
    adjoint.acoustic_pml_gradient(vp, d, dt, h, wavelet, [src], [rec], resid, order=order,
                                  dtype=np.float32)
    return time.perf_counter() - t0


def forward_one_shot(args):
    """Forward modelling of one shot (records), the oracle in float32."""
    vp, d, dt, h, wavelet, src, rec, order = args
    from oracle import fd2d
    t0 = time.perf_counter()
    fd2d.forward("acoustic", {"vp": vp}, d, dt, h, wavelet, [src], [rec], order=order, dtype=np.float32)
    return time.perf_counter() - t0


def acoustic_gradient_rate(vp, d, dt, h, wavelet, sources, receivers, order, nsteps, procs=None):
    """Run ``procs`` shots of ``nsteps`` steps in parallel processes.

    Returns (gpts_per_s, wall_s, procs)."""
    procs = procs or os.cpu_count() or 1
    procs = max(1, min(procs, len(sources)))
    w = np.asarray(wavelet[:nsteps], np.float32)
    jobs = [(vp, d, dt, h, w, sources[i], receivers[i], order) for i in range(procs)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        # warm the workers (interpreter start, numpy / oracle imports) outside the timed region
        pool.map(_one_shot, [(vp, d, dt, h, w[:2], sources[i], receivers[i], order) for i in range(procs)])
        t0 = time.perf_counter()
        pool.map(_one_shot, jobs)
        wall = time.perf_counter() - t0
    pts = procs * vp.size * nsteps
    return pts / wall / 1e9, wall, procs
