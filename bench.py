"""Benchmark of the seistorch hot path on GB300.

Workload (one "step" = one FWI gradient evaluation over one batch of shots):
2D acoustic L2-misfit adjoint gradient, 400 x 1000 interior + 50-cell PML
(500 x 1100 padded), dx = 10 m, dt = 1 ms, 3000 steps, 8th-order space,
fp32; vp a smooth random field 1500-4500 m/s (seeded N(0,1) noise, Gaussian
filter sigma = 20 cells, rescaled); 64 shots batched on row 2, 8 Hz Ricker,
1000 receivers on row 2; boundary-saving wavefield reconstruction.  The step
is forward (records) -> L2 residual against observed data (computed once from
the true model) -> fused adjoint -> dJ/dvp.

value  = shots * padded points * time steps / step time   [Gpts/s fwd+adjoint]
e2e    = the same through the public API (build_model / WaveRNN / autograd)
         with the model and observed data copied host->device and the
         gradient and loss copied back inside the timed region.
Inputs are larger than L2 (each wavefield buffer is 141 MB; ~25 GB resident).

--impl reference runs the CPU implementation of the same path (the oracle
port; the reference itself is Python on PyTorch and cannot run here) on the
host cores.  Multi-GPU (torchrun, --gpus N): shots are sharded, each rank
runs its own batch of 64 and the gradient is summed with one all-reduce.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NZI, NXI, WIDTH = 400, 1000, 50
DT, H, NT, ORDER, FM = 0.001, 10.0, 3000, 8, 8.0
NSHOTS, NREC = 64, 1000
WORKLOAD = "acoustic_l2_gradient_400x1000_pml50_o8_nt3000_64shots"
METRIC = "Gpts/s fwd+adjoint"
# algorithmic bytes per shot per padded point per time step (fp32)
BYTES_FWD = 12          # read U_n, U_{n-1}; write U_{n+1}
BYTES_BWD = 32          # reconstruction 12 + adjoint 12 + gradient accumulate 8
CPU_SAMPLE_STEPS = 200  # time steps per shot of the CPU sample (about 10 s of work per process)
BYTES_COEF = 8          # (g, k) planes, read once per point per step, shared by the shots


def make_models(seed=0):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    noise = gaussian_filter(rng.standard_normal((NZI, NXI)), sigma=20)
    noise = (noise - noise.min()) / (noise.max() - noise.min())
    vp_true = 1500.0 + 3000.0 * noise
    vp_init = gaussian_filter(vp_true, sigma=40)
    pad = lambda m: np.pad(m, WIDTH, mode="edge")
    return pad(vp_true), pad(vp_init)


def acquisition_lists():
    xs = np.linspace(0, NXI - 1, NSHOTS).round().astype(int)
    sources = [[(WIDTH + 2, WIDTH + int(x))] for x in xs]
    rx = list(range(WIDTH, WIDTH + NREC))
    receivers = [([WIDTH + 2] * NREC, rx)] * NSHOTS
    return sources, receivers


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu_index = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        with open(self.file.name) as f:
            rows = [r.strip().split(", ") for r in f if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """Per-launch DRAM bytes of the adjoint kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def cpu_baseline(vp, d, wavelet, sources, receivers, nsteps=40, procs=None):
    from oracle import baseline
    rate, wall, procs = baseline.acoustic_gradient_rate(vp, d, DT, H, wavelet, sources, receivers, ORDER,
                                                        nsteps, procs)
    return {"value": rate, "unit": "Gpts/s", "cores": procs, "kind": "port",
            "sample": f"{procs} shots x {nsteps} steps of the full 500x1100 o8 grid, forward+adjoint, "
                      f"numpy fp32, one process per shot ({wall:.1f} s wall)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import fd2d
    _, vp_init = make_models()
    d = fd2d.pml_profile_2d(vp_init.shape, WIDTH).astype(np.float32)
    wav = fd2d.ricker(FM, DT, NT, delay=int(1.2 / FM / DT))
    sources, receivers = acquisition_lists()
    nsteps = CPU_SAMPLE_STEPS
    vals = []
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_baseline(vp_init, d, wav, sources, receivers, nsteps=5)
    for _ in range(args.steps):
        vals.append(cpu_baseline(vp_init, d, wav, sources, receivers, nsteps=nsteps))
    rate = float(np.median([v["value"] for v in vals]))
    cb = dict(vals[-1])
    cb["value"] = rate
    step_s = NSHOTS * vp_init.size * NT / (rate * 1e9)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "Gpts/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "sample_steps_per_shot": nsteps},
            "cpu_baseline": cb,
            "e2e": {"value": rate, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    global NT, NSHOTS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--nt", type=int, default=NT)
    ap.add_argument("--shots", type=int, default=NSHOTS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    from seistorch_gb300 import _native, engine
    from seistorch_gb300.pml import generate_pml_coefficients_2d
    from seistorch_gb300.utils import ricker_wave

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _native.load(build_if_missing=False)

    NT, NSHOTS = args.nt, args.shots
    vp_true, vp_init = make_models(seed=0)
    nz, nx = vp_true.shape
    d = generate_pml_coefficients_2d((nz, nx), WIDTH).to(torch.float32).numpy()
    wav = ricker_wave(FM, DT, NT, delay=int(1.2 / FM / DT), dtype="numpy")
    sources, receivers = acquisition_lists()
    sources, receivers = sources[:NSHOTS], receivers[:NSHOTS]
    ckpt = engine.default_ckpt_every(NT)
    prop = engine.AcousticPropagator(nz, nx, DT, H, ORDER, "pml", WIDTH, False, dev)
    acq = engine.Acquisition(nz, nx, sources, receivers, wav, dev)
    d_t = torch.tensor(d, device=dev)
    with torch.no_grad():
        obs, _ = engine.acoustic_loop(torch.tensor(vp_true, dtype=torch.float32, device=dev), prop, d_t, acq)
    obs = obs.contiguous()
    vp_base = torch.tensor(vp_init, dtype=torch.float32, device=dev)

    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(timing=None):
        vp = vp_base.clone().requires_grad_(True)
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        rec, _ = engine.acoustic_loop(vp, prop, d_t, acq, False, ckpt)
        e1.record(stream)
        loss = ((rec - obs) ** 2).sum()
        loss.backward()
        if world > 1:
            dist.all_reduce(vp.grad)
        e2.record(stream)
        if timing is not None:
            timing.append((e0, e1, e2))
        return loss, vp.grad

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    timing = []
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t_start, t_end = ev(), ev()
        t_start.record(stream)
        for _ in range(args.steps):
            step(timing)
        t_end.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    total_ms = t_start.elapsed_time(t_end)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = t.item()
    ms_step = total_ms / args.steps
    pts = NSHOTS * nz * nx * NT * world
    value = pts / (ms_step * 1e-3) / 1e9
    fwd_ms = float(np.median([a.elapsed_time(b) for a, b, _ in timing]))
    bwd_ms = float(np.median([b.elapsed_time(c) for _, b, c in timing]))
    fwd_launch_ms = fwd_ms / NT
    bwd_launch_ms = bwd_ms / (NT - 1)
    npts = nz * nx
    bwd_bytes = NSHOTS * npts * BYTES_BWD + npts * BYTES_COEF
    fwd_bytes = NSHOTS * npts * BYTES_FWD + npts * BYTES_COEF
    peak, peak_kind = measured_peaks()
    achieved = bwd_bytes / (bwd_launch_ms * 1e-3) / 1e9
    traffic = profile_traffic().get("acoustic_bwd_tile_kernel_per_launch_bytes")
    line = {
        "metric": METRIC, "value": value, "unit": "Gpts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [nz, nx], "shots_per_gpu": NSHOTS, "nt": NT,
                   "order": ORDER, "ckpt_every": ckpt, "l2": "inputs larger than L2 (141 MB per field)",
                   "parallelism": f"shots x{world}"},
        "shots_per_s": NSHOTS * world / (ms_step * 1e-3),
        "phases_ms": {"forward": fwd_ms, "adjoint": bwd_ms},
        "roofline": {"kernel": "acoustic_bwd_tile_kernel", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "bytes_per_launch": bwd_bytes, "launch_ms": bwd_launch_ms},
        "roofline_forward": {"kernel": "acoustic_fwd_tile_kernel", "achieved": fwd_bytes / (fwd_launch_ms * 1e-3) / 1e9,
                             "frac": fwd_bytes / (fwd_launch_ms * 1e-3) / 1e9 / peak, "unit": "GB/s",
                             "launch_ms": fwd_launch_ms},
        "gpu_launches": args.steps * (NT + (NT - 1) + 2),
        "clocks": clocks.summary(),
    }
    if not args.no_e2e:
        line["e2e"] = e2e_through_api(args, dev, vp_init, obs.cpu(), wav, sources, receivers, world)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(vp_init, d, wav, sources, receivers, nsteps=CPU_SAMPLE_STEPS)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def e2e_through_api(args, dev, vp_init, obs_host, wav, sources, receivers, world):
    """Same metric through build_model / WaveRNN / autograd with host buffers."""
    import torch
    import torch.distributed as dist

    from seistorch_gb300 import build_model

    cfg = {"equation": "acoustic", "dtype": "float32",
           "geom": {"dt": DT, "h": H, "nt": NT, "boundary": {"type": "pml", "width": WIDTH},
                    "multiple": False, "boundary_saving": True, "source_type": ["h1"], "receiver_type": ["h1"],
                    "spatial_order": ORDER, "invlist": {"vp": True}}}
    vp_int = vp_init[WIDTH:-WIDTH, WIDTH:-WIDTH]
    _, model = build_model(cfg, device=dev, mode="inversion", models={"vp": vp_int})
    srcs = [[x - WIDTH, z - WIDTH] for [(z, x)] in sources]
    recs = [[[x - WIDTH for x in xs], [z - WIDTH for z in zs]] for zs, xs in receivers]
    model.reset_geom(list(range(len(srcs))), srcs, recs, cfg)
    vp_host = torch.tensor(vp_init, dtype=torch.float32).pin_memory()
    obs_pinned = obs_host.reshape(NT, len(sources), NREC).permute(1, 0, 2).contiguous().pin_memory()
    wav_host = torch.tensor(wav)[None].pin_memory()
    grad_host = torch.empty_like(vp_host).pin_memory()
    loss_host = torch.empty(1).pin_memory()
    param = model.cell.geom.vp

    def step():
        with torch.no_grad():
            param.copy_(vp_host.to(dev, non_blocking=True))
        param.grad = None
        obs = obs_pinned.to(dev, non_blocking=True)
        x = wav_host.to(dev, non_blocking=True)
        y = model(x)
        syn = torch.stack([t[..., 0] for t in y.data])  # (shots, nt, nrec)
        loss = ((syn - obs) ** 2).sum()
        loss.backward()
        if world > 1:
            dist.all_reduce(param.grad)
        grad_host.copy_(param.grad, non_blocking=True)
        loss_host.copy_(loss.detach().reshape(1), non_blocking=True)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    nz, nx = vp_init.shape
    h2d = vp_host.numel() * 4 + obs_pinned.numel() * 4 + wav_host.numel() * 4
    return {"value": len(sources) * nz * nx * NT * world / wall / 1e9, "unit": "Gpts/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(grad_host.numel() * 4 + 4),
            "ms_per_step": wall * 1e3, "api": "build_model -> WaveRNN.forward -> loss.backward"}


if __name__ == "__main__":
    sys.exit(main())
