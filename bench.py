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

--impl reference runs the CPU implementation of the same path on the host
cores: the oracle port (numpy fp32 restatement of the same discrete
algorithm, one process per shot), because the reference package itself is
not shipped with this repository.  On the same sample (8 shots x 40 steps of
this 500 x 1100, 8th-order grid, 8 CPU threads) the reference's own PyTorch
CPU path (WaveRNN with pure autograd) ran at 0.0036 Gpts/s and the port at
0.049 Gpts/s, so the port is the faster CPU baseline of the two (13.7x).  Multi-GPU (torchrun, --gpus N): shots are sharded, each rank
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
    ap.add_argument("--workload", default="acoustic_gradient",
                    choices=["acoustic_gradient", "elastic_gradient", "uneven_forward", "learned_fwi", "learned_net",
                             "born_gradient", "vti_gradient", "rho_gradient", "forward_small", "habc_gradient"],
                    help="acoustic_gradient (default, the headline line); elastic_gradient: 300x800 + 50 PML "
                         "elastic forward+adjoint; uneven_forward: 4 grid sizes x 64 shots in one launch per step; "
                         "born_gradient: least-squares RTM gradient (Born modelling, HABC); "
                         "vti_gradient: VTI (vti_habc2) vp / eps / delta gradient; "
                         "rho_gradient: variable-density (acoustic_rho_habc) vp / rho gradient; "
                         "forward_small: 128x256 + 50 PML, 4th order, 8 shots, 1000 steps, forward only "
                         "(L2-resident); habc_gradient: the headline grid and model with the hybrid absorbing "
                         "boundary (acoustic_habc), --order 2 (default) or 4")
    ap.add_argument("--order", type=int, default=0, help="habc_gradient: spatial order (2 or 4)")
    ap.add_argument("--pairs", type=int, default=800, help="learned_fwi: training pairs")
    ap.add_argument("--epochs", type=int, default=12, help="learned_fwi: training epochs")
    ap.add_argument("--iters", type=int, default=20, help="learned_fwi: FWI iterations")
    ap.add_argument("--save-net", default="", help="learned_fwi: write the trained parameters (.npz)")
    args = ap.parse_args()
    if args.workload == "learned_fwi":
        return bench_learned(args)
    if args.workload == "learned_net":
        return bench_net(args)
    if args.workload == "elastic_gradient":
        return bench_elastic(args)
    if args.workload == "uneven_forward":
        return bench_uneven(args)
    if args.workload == "born_gradient":
        return bench_born(args)
    if args.workload == "vti_gradient":
        return bench_vti(args)
    if args.workload == "rho_gradient":
        return bench_rho(args)
    if args.workload == "forward_small":
        return bench_forward_small(args)
    if args.workload == "habc_gradient":
        return bench_habc(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    from seistorch_gb300 import _native, engine
    from seistorch_gb300.distributed import allreduce_gradient
    from seistorch_gb300.postprocess import L2
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
        loss = L2()(rec, obs)
        loss.backward()
        if world > 1:
            allreduce_gradient(vp.grad)
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
        # the whole forward+adjoint step: 44 B per shot-point and time step
        # (forward 12 + reconstruction 12 + adjoint 12 + gradient 8) plus the
        # shared coefficient planes, over the step's wall time on the device
        "roofline_step": {"achieved": (fwd_bytes * NT + bwd_bytes * (NT - 1)) / (ms_step * 1e-3) / 1e9,
                          "frac": (fwd_bytes * NT + bwd_bytes * (NT - 1)) / (ms_step * 1e-3) / 1e9 / peak,
                          "unit": "GB/s", "bytes_per_step": fwd_bytes * NT + bwd_bytes * (NT - 1)},
        # per step: NT forward, NT-1 reverse, coefficients, misfit, gradient reduction
        "gpu_launches": args.steps * (NT + (NT - 1) + 3),
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


def e2e_through_api(args, dev, vp_init, obs_host, wav, sources, receivers, world, equation="acoustic",
                    boundary="pml", order=ORDER, nt=NT):
    """Same metric through build_model / WaveRNN / autograd with host buffers
    (`equation` acoustic with a PML, or acoustic_habc with the HABC)."""
    import torch
    import torch.distributed as dist

    from seistorch_gb300 import build_model
    from seistorch_gb300.distributed import allreduce_gradient
    from seistorch_gb300.postprocess import L2

    cfg = {"equation": equation, "dtype": "float32",
           "geom": {"dt": DT, "h": H, "nt": nt, "boundary": {"type": boundary, "width": WIDTH},
                    "multiple": False, "boundary_saving": True, "source_type": ["h1"], "receiver_type": ["h1"],
                    "spatial_order": order, "invlist": {"vp": True}}}
    vp_int = vp_init[WIDTH:-WIDTH, WIDTH:-WIDTH]
    _, model = build_model(cfg, device=dev, mode="inversion", models={"vp": vp_int})
    srcs = [[x - WIDTH, z - WIDTH] for [(z, x)] in sources]
    recs = [[[x - WIDTH for x in xs], [z - WIDTH for z in zs]] for zs, xs in receivers]
    model.reset_geom(list(range(len(srcs))), srcs, recs, cfg)
    vp_host = torch.tensor(vp_init, dtype=torch.float32).pin_memory()
    obs_pinned = obs_host.reshape(nt, len(sources), NREC).permute(1, 0, 2).contiguous().pin_memory()
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
        loss = L2()(syn, obs)
        loss.backward()
        if world > 1:
            allreduce_gradient(param.grad)
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
    return {"value": len(sources) * nz * nx * nt * world / wall / 1e9, "unit": "Gpts/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(grad_host.numel() * 4 + 4),
            "ms_per_step": wall * 1e3, "api": "build_model -> WaveRNN.forward -> loss.backward"}


# ------------------------------------------------- small forward (C1) ---
# 128 x 256 interior + 50-cell PML (228 x 356), dx = 10 m, dt = 1 ms, 1000
# steps, 4th order, fp32; vp: 3 horizontal layers 1500 / 2500 / 3500 m/s plus
# a Gaussian anomaly (+300 m/s, sigma = 10 cells, centre drawn from the seed);
# 8 shots on row 2 spaced 32 cells, 10 Hz Ricker, receivers on every cell of
# row 2.  One step = one forward modelling of the 8 shots (records).  The
# working set (three 2.6 MB fields) lives in L2, so the figure is reported
# against the HBM roofline for reference only.
FS_NZI, FS_NXI, FS_NT, FS_ORDER, FS_FM, FS_SHOTS = 128, 256, 1000, 4, 10.0, 8


def forward_small_case(seed=0):
    rng = np.random.default_rng(seed)
    vp = np.zeros((FS_NZI, FS_NXI))
    b = np.linspace(0, FS_NZI, 4).astype(int)
    for v, z0, z1 in zip((1500.0, 2500.0, 3500.0), b[:-1], b[1:]):
        vp[z0:z1] = v
    zz, xx = np.mgrid[0:FS_NZI, 0:FS_NXI]
    cz, cx = rng.uniform(0.3, 0.7) * FS_NZI, rng.uniform(0.3, 0.7) * FS_NXI
    vp += 300.0 * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * 10.0 ** 2))
    vp = np.pad(vp, WIDTH, mode="edge")
    sources = [[(WIDTH + 2, WIDTH + 16 + 32 * k)] for k in range(FS_SHOTS)]
    receivers = [([WIDTH + 2] * FS_NXI, list(range(WIDTH, WIDTH + FS_NXI)))] * FS_SHOTS
    return vp, sources, receivers


def cpu_forward_rate(vp, d, wav, sources, receivers, procs=None):
    """The oracle port (numpy fp32) of the same forward, one process per shot."""
    import multiprocessing as mp
    from oracle import baseline
    procs = max(1, min(procs or os.cpu_count() or 1, len(sources)))
    jobs = [(vp, d, DT, H, wav, sources[i], receivers[i], FS_ORDER) for i in range(len(sources))]
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        pool.map(baseline.forward_one_shot, [(vp, d, DT, H, wav[:2], sources[0], receivers[0], FS_ORDER)] * procs)
        t0 = time.perf_counter()
        pool.map(baseline.forward_one_shot, jobs)
        wall = time.perf_counter() - t0
    return len(sources) * vp.size * len(wav) / wall / 1e9, wall, procs


def bench_forward_small(args):
    from oracle import fd2d
    vp, sources, receivers = forward_small_case()
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), WIDTH).astype(np.float32)
    wav = fd2d.ricker(FS_FM, DT, FS_NT, delay=int(1.0 / FS_FM / DT))
    metric, unit = "Gpts/s fwd", "Gpts/s"
    config = {"workload": "acoustic_forward_128x256_pml50_o4_nt1000_8shots", "grid": [nz, nx], "shots": FS_SHOTS,
              "nt": FS_NT, "order": FS_ORDER, "l2": "L2-resident (2.6 MB per field); not an HBM-bound case"}
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return 0
        vals = [cpu_forward_rate(vp, d, wav, sources, receivers) for _ in range(max(1, args.steps))]
        rate = float(np.median([v[0] for v in vals]))
        cb = {"value": rate, "unit": unit, "cores": vals[-1][2], "kind": "port",
              "sample": f"the whole workload ({FS_SHOTS} shots x {FS_NT} steps), numpy fp32, one process per shot"}
        print(json.dumps({"impl": "reference", "metric": metric, "value": rate, "unit": unit, "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": FS_SHOTS * nz * nx * FS_NT / (rate * 1e9) * 1e3,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic", "config": config, "cpu_baseline": cb,
                          "e2e": {"value": rate, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return 0
    import torch
    from seistorch_gb300 import _native, build_model, engine
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    prop = engine.AcousticPropagator(nz, nx, DT, H, FS_ORDER, "pml", WIDTH, False, dev)
    acq = engine.Acquisition(nz, nx, sources, receivers, wav, dev)
    vpt = torch.tensor(vp, dtype=torch.float32, device=dev)
    dt_ = torch.tensor(d, device=dev)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    with torch.no_grad():
        for _ in range(max(3, args.warmup)):
            engine.acoustic_loop(vpt, prop, dt_, acq)
        torch.cuda.synchronize()
        with ClockSampler(0) as clocks:
            t0, t1 = ev(), ev()
            t0.record(stream)
            for _ in range(args.steps):
                engine.acoustic_loop(vpt, prop, dt_, acq)
            t1.record(stream)
            torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    pts = FS_SHOTS * nz * nx * FS_NT
    peak, kind = measured_peaks()
    gbs = (FS_SHOTS * nz * nx * BYTES_FWD + nz * nx * BYTES_COEF) * FS_NT / (ms * 1e-3) / 1e9
    # end to end: build_model -> WaveRNN.forward with the model copied in and the records copied out
    cfg = {"equation": "acoustic", "dtype": "float32",
           "geom": {"dt": DT, "h": H, "nt": FS_NT, "boundary": {"type": "pml", "width": WIDTH}, "multiple": False,
                    "source_type": ["h1"], "receiver_type": ["h1"], "spatial_order": FS_ORDER}}
    _, model = build_model(cfg, device=dev, mode="forward", models={"vp": vp[WIDTH:-WIDTH, WIDTH:-WIDTH]})
    srcs = [[x - WIDTH, z - WIDTH] for [(z, x)] in sources]
    recs = [[[x - WIDTH for x in xs], [z - WIDTH for z in zs]] for zs, xs in receivers]
    model.reset_geom(list(range(FS_SHOTS)), srcs, recs, cfg)
    vp_host = torch.tensor(vp, dtype=torch.float32).pin_memory()
    wav_host = torch.tensor(wav)[None].pin_memory()
    rec_host = torch.empty(FS_SHOTS, FS_NT, FS_NXI).pin_memory()
    param = model.cell.geom.vp

    def api_step():
        with torch.no_grad():
            param.copy_(vp_host.to(dev, non_blocking=True))
            y = model(wav_host.to(dev, non_blocking=True))
            rec_host.copy_(torch.stack([t[..., 0] for t in y.data]), non_blocking=True)

    for _ in range(max(3, args.warmup)):
        api_step()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        api_step()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - w0) / args.steps
    line = {"metric": metric, "value": pts / (ms * 1e-3) / 1e9, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
            "shots_per_s": FS_SHOTS / (ms * 1e-3),
            "roofline": {"kernel": "acoustic_fwd_tile_kernel", "bound": "hbm", "achieved": gbs, "peak": peak,
                         "peak_kind": kind, "unit": "GB/s", "frac": gbs / peak, "traffic": None,
                         "note": "working set in L2: the HBM bound does not apply; shown for comparison"},
            "gpu_launches": args.steps * (FS_NT + 1), "clocks": clocks.summary(),
            "e2e": {"value": pts / wall / 1e9, "unit": unit, "h2d_bytes_per_step": int(vp_host.numel() * 4 +
                                                                                          wav_host.numel() * 4),
                    "d2h_bytes_per_step": int(rec_host.numel() * 4), "ms_per_step": wall * 1e3,
                    "api": "build_model -> WaveRNN.forward (records to host)"}}
    if not args.no_cpu_baseline:
        rate, wall_c, procs = cpu_forward_rate(vp, d, wav, sources, receivers)
        line["cpu_baseline"] = {"value": rate, "unit": unit, "cores": procs, "kind": "port",
                                "sample": f"the whole workload ({FS_SHOTS} shots x {FS_NT} steps), numpy fp32, "
                                          f"one process per shot ({wall_c:.1f} s wall)"}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------- HABC ---
# acoustic_habc gradient: the headline grid, model and acquisition (400 x
# 1000 interior + 50-cell hybrid absorbing boundary, dx = 10 m, dt = 1 ms,
# 3000 steps, 64 shots, 8 Hz, 1000 receivers on row 2), 2nd order (the
# reference's default) or 4th.  One step = forward + L2 residual against data
# from the true model + HABC adjoint (tiled interior + frame kernels) + dJ/dvp.
HB_BYTES_FWD, HB_BYTES_REV, HB_BYTES_COEF = 12, 32, 8


def bench_habc(args):
    import torch
    from seistorch_gb300 import _native, engine
    from seistorch_gb300.habc import generate_habc_coefficients_2d
    from seistorch_gb300.postprocess import L2
    from seistorch_gb300.utils import ricker_wave
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the acoustic "
                          "gradient workload only"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    order = args.order or 2
    nt, shots = args.nt, args.shots
    vp_true, vp_init = make_models(seed=0)
    nz, nx = vp_true.shape
    b = generate_habc_coefficients_2d((nz, nx), WIDTH).to(device=dev, dtype=torch.float32)
    wav = ricker_wave(FM, DT, nt, delay=int(1.2 / FM / DT), dtype="numpy")
    sources, receivers = acquisition_lists()
    sources, receivers = sources[:shots], receivers[:shots]
    prop = engine.AcousticPropagator(nz, nx, DT, H, order, "habc", WIDTH, False, dev)
    acq = engine.Acquisition(nz, nx, sources, receivers, wav, dev)
    t = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    ck = engine.default_ckpt_every(nt)
    with torch.no_grad():
        obs, _ = engine.acoustic_loop(t(vp_true), prop, b, acq)
    obs = obs.contiguous()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(timing=None):
        vp = t(vp_init, True)
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        r, _ = engine.acoustic_loop(vp, prop, b, acq, False, ck)
        e1.record(stream)
        loss = L2()(r, obs)
        loss.backward()
        e2.record(stream)
        if timing is not None:
            timing.append((e0, e1, e2))
        return loss

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    timing = []
    with ClockSampler(0) as clocks:
        t0, t1 = ev(), ev()
        t0.record(stream)
        for _ in range(args.steps):
            step(timing)
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    fwd_ms = float(np.median([a.elapsed_time(c) for a, c, _ in timing]))
    rev_ms = float(np.median([c.elapsed_time(e) for _, c, e in timing]))
    npts = nz * nx
    rev_bytes = shots * npts * HB_BYTES_REV + npts * HB_BYTES_COEF
    fwd_bytes = shots * npts * HB_BYTES_FWD + npts * HB_BYTES_COEF
    peak, kind = measured_peaks()
    rev_gbs = rev_bytes / (rev_ms / (nt - 1) * 1e-3) / 1e9
    fwd_gbs = fwd_bytes / (fwd_ms / nt * 1e-3) / 1e9
    line = {"metric": "Gpts/s fwd+adjoint", "value": shots * npts * nt / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"acoustic_habc_l2_gradient_{NZI}x{NXI}_habc{WIDTH}_o{order}_nt{nt}_{shots}shots",
                       "grid": [nz, nx], "shots": shots, "nt": nt, "order": order, "ckpt_every": ck,
                       "l2": "inputs larger than L2 (141 MB per field)"},
            "shots_per_s": shots / (ms * 1e-3), "phases_ms": {"forward": fwd_ms, "adjoint": rev_ms},
            "roofline": {"kernel": "habc_bwd_tile_kernel (far + near tiles)", "bound": "hbm", "achieved": rev_gbs,
                         "peak": peak, "peak_kind": kind, "unit": "GB/s", "frac": rev_gbs / peak, "traffic": None,
                         "bytes_per_launch": rev_bytes, "launch_ms": rev_ms / (nt - 1)},
            "roofline_forward": {"kernel": "acoustic_fwd_tile_kernel<HABC>", "achieved": fwd_gbs,
                                 "frac": fwd_gbs / peak, "unit": "GB/s", "launch_ms": fwd_ms / nt},
            # per step: NT forward, 2 (NT-1) reverse (far and near tiles), share planes, coefficients,
            # misfit, reduction
            "gpu_launches": args.steps * (nt + 2 * (nt - 1) + 4), "clocks": clocks.summary()}
    if not args.no_e2e:
        line["e2e"] = e2e_through_api(args, dev, vp_init, obs.cpu(), wav, sources, receivers, 1,
                                      equation="acoustic_habc", boundary="habc", order=order, nt=nt)
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------ elastic ---
# 300 x 800 interior + 50-cell PML (400 x 900), dx = 5 m, dt = 0.5 ms, 4000
# steps; vp 2000-5000 m/s layered with a seeded dipping fault, vs = vp/1.73,
# rho = 310 vp^0.25; 32 explosive shots (txx + tzz) on row 2, 12 Hz Ricker,
# vx / vz receivers on every interior cell of row 2.  One step = forward +
# L2 residual against data from the true model + fused adjoint + dJ/d(vp,
# vs, rho).
EL_NZI, EL_NXI, EL_W, EL_DT, EL_H, EL_NT, EL_FM, EL_SHOTS = 300, 800, 50, 0.0005, 5.0, 4000, 12.0, 32
EL_BYTES_FWD = 40    # read 5 fields, write 5 fields
EL_BYTES_REV = 104   # read s, a (10 fields) + 3 gradient terms, write s, a + 3 gradient terms
EL_BYTES_COEF = 24   # 6 coefficient planes, shared by the shots


def elastic_models(seed=0):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    nl = 6
    tops = np.sort(rng.choice(np.arange(20, EL_NZI - 20), nl - 1, replace=False))
    vel = np.linspace(2000.0, 5000.0, nl) + rng.uniform(-150, 150, nl)
    zz, xx = np.mgrid[0:EL_NZI, 0:EL_NXI]
    x_f = EL_NXI * rng.uniform(0.35, 0.65)
    throw = int(rng.integers(15, 40))
    fault = (xx - x_f) > (zz - EL_NZI / 2) * 0.6  # dipping fault plane
    depth = np.where(fault, zz - throw, zz)
    layer = np.searchsorted(tops, depth, side="right")
    vp = np.clip(vel[layer], 2000.0, 5000.0)
    vp0 = gaussian_filter(vp, sigma=15)
    pad = lambda m: np.pad(m, EL_W, mode="edge")
    out = []
    for v in (vp, vp0):
        v = pad(v)
        out.append({"vp": v, "vs": v / 1.73, "rho": 310.0 * v ** 0.25})
    return out


def bench_elastic(args):
    import torch
    from seistorch_gb300 import _native, elastic_engine, engine
    from seistorch_gb300.pml import generate_pml_coefficients_2d
    from seistorch_gb300.postprocess import L2
    from seistorch_gb300.utils import ricker_wave
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the acoustic "
                          "gradient workload only"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    nt = args.nt if args.nt != NT else EL_NT
    shots = args.shots if args.shots != NSHOTS else EL_SHOTS
    true_m, init_m = elastic_models()
    nz, nx = true_m["vp"].shape
    d = generate_pml_coefficients_2d((nz, nx), EL_W).to(torch.float32)
    wav = ricker_wave(EL_FM, EL_DT, nt, delay=int(1.2 / EL_FM / EL_DT), dtype="numpy")
    xs = np.linspace(0, EL_NXI - 1, shots).round().astype(int)
    src = [[(EL_W + 2, EL_W + int(x))] for x in xs]
    rec = [([EL_W + 2] * EL_NXI, list(range(EL_W, EL_W + EL_NXI)))] * shots
    prop = elastic_engine.ElasticPropagator(nz, nx, EL_DT, EL_H, EL_W, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    io, nch = elastic_engine.make_io(["txx", "tzz"], ["vx", "vz"])
    t = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    dd = d.to(dev)
    ck = engine.default_ckpt_every(nt)
    with torch.no_grad():
        obs, _ = elastic_engine.elastic_records(t(true_m["vp"]), t(true_m["vs"]), t(true_m["rho"]), prop, dd,
                                                acq, io, nch)
    obs = obs.contiguous()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(timing=None):
        m = [t(init_m[k], True) for k in ("vp", "vs", "rho")]
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        r, _ = elastic_engine.elastic_records(*m, prop, dd, acq, io, nch, False, ck)
        e1.record(stream)
        loss = L2()(r, obs)
        loss.backward()
        e2.record(stream)
        if timing is not None:
            timing.append((e0, e1, e2))
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    timing = []
    with ClockSampler(0) as clocks:
        t0, t1 = ev(), ev()
        t0.record(stream)
        for _ in range(args.steps):
            step(timing)
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    fwd_ms = float(np.median([a.elapsed_time(b) for a, b, _ in timing]))
    rev_ms = float(np.median([b.elapsed_time(c) for _, b, c in timing]))
    npts = nz * nx
    rev_bytes = shots * npts * EL_BYTES_REV + npts * EL_BYTES_COEF
    fwd_bytes = shots * npts * EL_BYTES_FWD + npts * EL_BYTES_COEF
    peak, kind = measured_peaks()
    rev_gbs = rev_bytes / (rev_ms / nt * 1e-3) / 1e9
    fwd_gbs = fwd_bytes / (fwd_ms / nt * 1e-3) / 1e9
    line = {"metric": "Gpts/s fwd+adjoint", "value": shots * npts * nt / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"elastic_l2_gradient_{EL_NZI}x{EL_NXI}_pml{EL_W}_nt{nt}_{shots}shots",
                       "grid": [nz, nx], "shots": shots, "nt": nt, "ckpt_every": ck,
                       "l2": "inputs larger than L2 (46 MB per field, 5 fields)"},
            "shots_per_s": shots / (ms * 1e-3), "phases_ms": {"forward": fwd_ms, "adjoint": rev_ms},
            "roofline": {"kernel": "elastic_bwd_kernel", "bound": "hbm", "achieved": rev_gbs, "peak": peak,
                         "peak_kind": kind, "unit": "GB/s", "frac": rev_gbs / peak, "traffic": None,
                         "bytes_per_launch": rev_bytes, "launch_ms": rev_ms / nt},
            "roofline_forward": {"kernel": "elastic_fwd_kernel", "achieved": fwd_gbs, "frac": fwd_gbs / peak,
                                 "unit": "GB/s", "launch_ms": fwd_ms / nt},
            "gpu_launches": args.steps * (2 * nt + 2), "clocks": clocks.summary()}
    if not args.no_e2e:
        line["e2e"] = e2e_models(args, dev, "elastic", "pml", EL_W, EL_DT, EL_H, 2, dict(init_m),
                                 ("vp", "vs", "rho"), obs.cpu(), 2, wav, src, rec, nt, ["txx", "tzz"], ["vx", "vz"])
    print(json.dumps(line))
    return 0


def e2e_models(args, dev, equation, boundary, w, dt, h, order, models, inverted, obs_host, nch, wav, src, rec, nt,
               src_type, rec_type):
    """A gradient workload through build_model / WaveRNN / autograd: every
    step copies the padded models and the observed data from pinned host
    memory, runs WaveRNN.forward and loss.backward, and copies the inverted
    models' gradients and the loss back.  models: name -> padded array;
    inverted: the names whose gradient is taken; obs_host: (nt, shots x nrec,
    nch) records of the true model."""
    import torch

    from seistorch_gb300 import build_model
    from seistorch_gb300.postprocess import L2

    names = list(models)
    cfg = {"equation": equation, "dtype": "float32",
           "geom": {"dt": dt, "h": h, "nt": nt, "boundary": {"type": boundary, "width": w},
                    "multiple": False, "boundary_saving": True, "source_type": list(src_type),
                    "receiver_type": list(rec_type), "spatial_order": order,
                    "invlist": {k: k in inverted for k in names}}}
    _, model = build_model(cfg, device=dev, mode="inversion",
                           models={k: np.asarray(models[k])[w:-w, w:-w] for k in names})
    srcs = [[x - w, z - w] for [(z, x)] in src]
    recs = [[[x - w for x in xs], [z - w for z in zs]] for zs, xs in rec]
    model.reset_geom(list(range(len(srcs))), srcs, recs, cfg)
    shots, nrec = len(src), len(rec[0][0])
    hosts = {k: torch.tensor(np.asarray(models[k]), dtype=torch.float32).pin_memory() for k in names}
    obs_pinned = obs_host.reshape(nt, shots, nrec, nch).permute(1, 0, 2, 3).contiguous().pin_memory()
    wav_host = torch.tensor(wav)[None].pin_memory()
    grads_host = {k: torch.empty_like(hosts[k]).pin_memory() for k in inverted}
    loss_host = torch.empty(1).pin_memory()
    params = {k: getattr(model.cell.geom, k) for k in names}

    def step():
        with torch.no_grad():
            for k in names:
                params[k].copy_(hosts[k].to(dev, non_blocking=True))
        for k in inverted:
            params[k].grad = None
        obs = obs_pinned.to(dev, non_blocking=True)
        y = model(wav_host.to(dev, non_blocking=True))
        loss = L2()(torch.stack(list(y.data)), obs)
        loss.backward()
        for k in inverted:
            grads_host[k].copy_(params[k].grad, non_blocking=True)
        loss_host.copy_(loss.detach().reshape(1), non_blocking=True)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    nz, nx = hosts[names[0]].shape
    h2d = sum(t_.numel() for t_ in hosts.values()) * 4 + obs_pinned.numel() * 4 + wav_host.numel() * 4
    return {"value": shots * nz * nx * nt / wall / 1e9, "unit": "Gpts/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(sum(t_.numel() for t_ in grads_host.values()) * 4 + 4),
            "ms_per_step": wall * 1e3, "api": "build_model -> WaveRNN.forward -> loss.backward"}


# --------------------------------------------------------------- Born ---
# Least-squares RTM gradient (acoustic_lsrtm_habc, examples/lsrtm/acoustic):
# 400 x 1000 interior + 50-cell HABC (500 x 1100), dx = 10 m, dt = 1 ms,
# 2000 steps, 2nd order (the equation module's spatial_order); smoothed
# layered background vp 1500-3500 m/s held fixed; true reflectivity
# m = 2 dv / v0 of the layered model, the gradient taken at half of it;
# 32 shots on row 2, 10 Hz Ricker, receivers on every interior cell of row 2
# recording the scattered field.  One step = Born forward (background +
# scattered fields) + L2 residual + HABC adjoint + dJ/dm.
BN_NZI, BN_NXI, BN_W, BN_DT, BN_H, BN_NT, BN_FM, BN_SHOTS = 400, 1000, 50, 0.001, 10.0, 2000, 10.0, 32
BN_BYTES_FWD = 32  # background: read p, p-, write p+, m k L(p); scattered: read s, s-, m k L(p), write s+
BN_BYTES_REV = 32  # read La1, La2, U_j, U_{j-1}, grad; write La_j, U_{j-2}, grad
BN_BYTES_COEF = 16  # vp, blend weight, g / k, m planes, shared by the shots


def born_models(seed=0):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    nl = 7
    tops = np.sort(rng.choice(np.arange(20, BN_NZI - 20), nl - 1, replace=False))
    vel = np.linspace(1500.0, 3500.0, nl) + rng.uniform(-100, 100, nl)
    zz, xx = np.mgrid[0:BN_NZI, 0:BN_NXI]
    depth = zz + (8.0 * np.sin(2 * np.pi * xx / BN_NXI * rng.uniform(1, 3))).astype(int)
    vp = vel[np.searchsorted(tops, depth, side="right")]
    v0 = gaussian_filter(vp, sigma=12)
    m_true = 2.0 * (vp - v0) / v0
    pad = lambda a: np.pad(a, BN_W, mode="edge")
    return pad(v0), pad(m_true)


def bench_born(args):
    import torch
    from seistorch_gb300 import _native, engine
    from seistorch_gb300.habc import generate_habc_coefficients_2d
    from seistorch_gb300.postprocess import L2
    from seistorch_gb300.utils import ricker_wave
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the acoustic "
                          "gradient workload only"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    nt = args.nt if args.nt != NT else BN_NT
    shots = args.shots if args.shots != NSHOTS else BN_SHOTS
    v0, m_true = born_models()
    nz, nx = v0.shape
    b = generate_habc_coefficients_2d((nz, nx), BN_W).to(torch.float32)
    wav = ricker_wave(BN_FM, BN_DT, nt, delay=int(1.2 / BN_FM / BN_DT), dtype="numpy")
    xs = np.linspace(0, BN_NXI - 1, shots).round().astype(int)
    src = [[(BN_W + 2, BN_W + int(x))] for x in xs]
    rec = [([BN_W + 2] * BN_NXI, list(range(BN_W, BN_W + BN_NXI)))] * shots
    prop = engine.BornPropagator(nz, nx, BN_DT, BN_H, 2, BN_W, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    t = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    vp, bb = t(v0), b.to(dev)
    ck = engine.default_ckpt_every(nt)
    with torch.no_grad():
        obs = engine.born_loop(vp, t(m_true), prop, bb, acq).contiguous()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(timing=None):
        m = t(0.5 * m_true, True)
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        r = engine.born_loop(vp, m, prop, bb, acq, ck)
        e1.record(stream)
        loss = L2()(r, obs)
        loss.backward()
        e2.record(stream)
        if timing is not None:
            timing.append((e0, e1, e2))
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    timing = []
    with ClockSampler(0) as clocks:
        t0, t1 = ev(), ev()
        t0.record(stream)
        for _ in range(args.steps):
            step(timing)
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    fwd_ms = float(np.median([a.elapsed_time(c) for a, c, _ in timing]))
    rev_ms = float(np.median([c.elapsed_time(e) for _, c, e in timing]))
    npts = nz * nx
    rev_bytes = shots * npts * BN_BYTES_REV + npts * BN_BYTES_COEF
    fwd_bytes = shots * npts * BN_BYTES_FWD + npts * BN_BYTES_COEF
    peak, kind = measured_peaks()
    rev_gbs = rev_bytes / (rev_ms / (nt - 1) * 1e-3) / 1e9
    fwd_gbs = fwd_bytes / (fwd_ms / nt * 1e-3) / 1e9
    line = {"metric": "Gpts/s fwd+adjoint", "value": shots * npts * nt / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"born_lsrtm_gradient_{BN_NZI}x{BN_NXI}_habc{BN_W}_o2_nt{nt}_{shots}shots",
                       "grid": [nz, nx], "shots": shots, "nt": nt, "ckpt_every": ck,
                       "l2": "inputs larger than L2 (70 MB per field, 6 fields)"},
            "shots_per_s": shots / (ms * 1e-3), "phases_ms": {"forward": fwd_ms, "adjoint": rev_ms},
            "roofline": {"kernel": "habc_bwd_tile_kernel (far + near tiles)", "bound": "hbm", "achieved": rev_gbs, "peak": peak,
                         "peak_kind": kind, "unit": "GB/s", "frac": rev_gbs / peak, "traffic": None,
                         "bytes_per_launch": rev_bytes, "launch_ms": rev_ms / (nt - 1)},
            "roofline_forward": {"kernel": "acoustic_fwd_tile_kernel<HABC> x2 (background, scattered)",
                                 "achieved": fwd_gbs, "frac": fwd_gbs / peak, "unit": "GB/s",
                                 "launch_ms": fwd_ms / nt},
            # per step: 2 NT forward (background, scattered), 2 (NT-1) reverse (far and near tiles), share
            # planes, coefficients, misfit, reduction
            "gpu_launches": args.steps * (2 * nt + 2 * (nt - 1) + 4), "clocks": clocks.summary()}
    if not args.no_e2e:
        line["e2e"] = e2e_models(args, dev, "acoustic_lsrtm_habc", "habc", BN_W, BN_DT, BN_H, 2,
                                 {"vp": v0, "m": 0.5 * m_true}, ("m",), obs.cpu(), 1, wav, src, rec, nt,
                                 ["h1"], ["sh1"])
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- VTI ---
# VTI gradient (vti_habc2): the Born grid and geometry above (400 x 1000 +
# 50-cell HABC, 2nd order, 2000 steps, 32 shots, receivers on row 2), the
# layered vp with eps = 0.1-0.25 and delta = 0.05-0.12 following the layers;
# L2 residual against data from the true model, gradient at the smoothed
# model (vp, eps, delta).  One step = forward + residual + adjoint + dJ/d(vp,
# eps, delta).
def bench_vti(args):
    import torch
    from scipy.ndimage import gaussian_filter
    from seistorch_gb300 import _native, engine
    from seistorch_gb300.habc import generate_habc_coefficients_2d
    from seistorch_gb300.postprocess import L2
    from seistorch_gb300.utils import ricker_wave
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the acoustic "
                          "gradient workload only"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    nt = args.nt if args.nt != NT else BN_NT
    shots = args.shots if args.shots != NSHOTS else BN_SHOTS
    v0, m_true = born_models()
    vp_true = v0 * (1.0 + 0.5 * m_true)  # layered velocity of the Born model
    eps_true = 0.1 + 0.15 * (vp_true - vp_true.min()) / (vp_true.max() - vp_true.min())
    delta_true = 0.05 + 0.07 * (vp_true - vp_true.min()) / (vp_true.max() - vp_true.min())
    init = [gaussian_filter(a, sigma=12) for a in (vp_true, eps_true, delta_true)]
    nz, nx = v0.shape
    b = generate_habc_coefficients_2d((nz, nx), BN_W).to(torch.float32)
    wav = ricker_wave(BN_FM, BN_DT, nt, delay=int(1.2 / BN_FM / BN_DT), dtype="numpy")
    xs = np.linspace(0, BN_NXI - 1, shots).round().astype(int)
    src = [[(BN_W + 2, BN_W + int(x))] for x in xs]
    rec = [([BN_W + 2] * BN_NXI, list(range(BN_W, BN_W + BN_NXI)))] * shots
    prop = engine.VTIPropagator(nz, nx, BN_DT, BN_H, BN_W, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    t = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    bb = b.to(dev)
    ck = engine.default_ckpt_every(nt)
    with torch.no_grad():
        obs = engine.vti_loop(t(vp_true), t(eps_true), t(delta_true), prop, bb, acq).contiguous()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(timing=None):
        ms = [t(a, True) for a in init]
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        r = engine.vti_loop(*ms, prop, bb, acq, ck)
        e1.record(stream)
        loss = L2()(r, obs)
        loss.backward()
        e2.record(stream)
        if timing is not None:
            timing.append((e0, e1, e2))
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    timing = []
    with ClockSampler(0) as clocks:
        t0, t1 = ev(), ev()
        t0.record(stream)
        for _ in range(args.steps):
            step(timing)
        t1.record(stream)
        torch.cuda.synchronize()
    ms_ = t0.elapsed_time(t1) / args.steps
    fwd_ms = float(np.median([a.elapsed_time(c) for a, c, _ in timing]))
    rev_ms = float(np.median([c.elapsed_time(e) for _, c, e in timing]))
    npts = nz * nx
    fwd_bytes = shots * npts * 12 + npts * 20   # read u, u-, write u+; g, kx, kz, vp, b planes
    rev_bytes = shots * npts * 36 + npts * 20   # read La1, La2, U_j, U_{j-1}, 2 gradients; write La_j, U_{j-2}, 2 gradients
    peak, kind = measured_peaks()
    rev_gbs = rev_bytes / (rev_ms / (nt - 1) * 1e-3) / 1e9
    fwd_gbs = fwd_bytes / (fwd_ms / nt * 1e-3) / 1e9
    line = {"metric": "Gpts/s fwd+adjoint", "value": shots * npts * nt / (ms_ * 1e-3) / 1e9, "unit": "Gpts/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"vti_l2_gradient_{BN_NZI}x{BN_NXI}_habc{BN_W}_o2_nt{nt}_{shots}shots",
                       "grid": [nz, nx], "shots": shots, "nt": nt, "ckpt_every": ck,
                       "l2": "inputs larger than L2 (70 MB per field)"},
            "shots_per_s": shots / (ms_ * 1e-3), "phases_ms": {"forward": fwd_ms, "adjoint": rev_ms},
            "roofline": {"kernel": "habc_bwd_tile_kernel (VTI, far + near tiles)", "bound": "hbm", "achieved": rev_gbs, "peak": peak,
                         "peak_kind": kind, "unit": "GB/s", "frac": rev_gbs / peak, "traffic": None,
                         "bytes_per_launch": rev_bytes, "launch_ms": rev_ms / (nt - 1)},
            "roofline_forward": {"kernel": "acoustic_fwd_tile_kernel<HABC> (VTI)", "achieved": fwd_gbs,
                                 "frac": fwd_gbs / peak, "unit": "GB/s", "launch_ms": fwd_ms / nt},
            # per step: NT forward, 2 (NT-1) reverse (far and near tiles), share planes, coefficients,
            # misfit, 2 reductions
            "gpu_launches": args.steps * (nt + 2 * (nt - 1) + 5), "clocks": clocks.summary()}
    if not args.no_e2e:
        line["e2e"] = e2e_models(args, dev, "vti_habc2", "habc", BN_W, BN_DT, BN_H, 2,
                                 dict(zip(("vp", "epsilon", "delta"), init)), ("vp", "epsilon", "delta"),
                                 obs.cpu(), 1, wav, src, rec, nt, ["p1"], ["p1"])
    print(json.dumps(line))
    return 0


# ---------------------------------------------------- variable density ---
# acoustic_rho_habc gradient: the Born grid and geometry (400 x 1000 + 50
# HABC, 2nd order, 2000 steps, 32 shots), the layered vp and a Gardner
# density rho = 310 vp^0.25; L2 residual against data from the true model,
# gradient at the smoothed model (vp, rho).
def bench_rho(args):
    import torch
    from scipy.ndimage import gaussian_filter
    from seistorch_gb300 import _native, engine
    from seistorch_gb300.habc import generate_habc_coefficients_2d
    from seistorch_gb300.postprocess import L2
    from seistorch_gb300.utils import ricker_wave
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the acoustic "
                          "gradient workload only"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    nt = args.nt if args.nt != NT else BN_NT
    shots = args.shots if args.shots != NSHOTS else BN_SHOTS
    v0, m_true = born_models()
    vp_true = v0 * (1.0 + 0.5 * m_true)
    rho_true = 310.0 * vp_true ** 0.25
    init = [gaussian_filter(a, sigma=12) for a in (vp_true, rho_true)]
    nz, nx = v0.shape
    b = generate_habc_coefficients_2d((nz, nx), BN_W).to(torch.float32)
    wav = ricker_wave(BN_FM, BN_DT, nt, delay=int(1.2 / BN_FM / BN_DT), dtype="numpy")
    xs = np.linspace(0, BN_NXI - 1, shots).round().astype(int)
    src = [[(BN_W + 2, BN_W + int(x))] for x in xs]
    rec = [([BN_W + 2] * BN_NXI, list(range(BN_W, BN_W + BN_NXI)))] * shots
    prop = engine.RhoPropagator(nz, nx, BN_DT, BN_H, BN_W, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    t = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    bb = b.to(dev)
    ck = engine.default_ckpt_every(nt)
    with torch.no_grad():
        obs = engine.rho_loop(t(vp_true), t(rho_true), prop, bb, acq).contiguous()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def step(timing=None):
        ms = [t(a, True) for a in init]
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        r = engine.rho_loop(*ms, prop, bb, acq, ck)
        e1.record(stream)
        loss = L2()(r, obs)
        loss.backward()
        e2.record(stream)
        if timing is not None:
            timing.append((e0, e1, e2))
        return loss

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    timing = []
    with ClockSampler(0) as clocks:
        t0, t1 = ev(), ev()
        t0.record(stream)
        for _ in range(args.steps):
            step(timing)
        t1.record(stream)
        torch.cuda.synchronize()
    ms_ = t0.elapsed_time(t1) / args.steps
    fwd_ms = float(np.median([a.elapsed_time(c) for a, c, _ in timing]))
    rev_ms = float(np.median([c.elapsed_time(e) for _, c, e in timing]))
    npts = nz * nx
    fwd_bytes = shots * npts * 12 + npts * 32   # read u, u-, write u+; g, C, 4 buoyancy, vp, b planes
    rev_bytes = shots * npts * 64 + npts * 32   # read La1, La2, U_j, U_{j-1}; write La_j, U_{j-2}; 5 gradients r/w
    peak, kind = measured_peaks()
    rev_gbs = rev_bytes / (rev_ms / (nt - 1) * 1e-3) / 1e9
    fwd_gbs = fwd_bytes / (fwd_ms / nt * 1e-3) / 1e9
    line = {"metric": "Gpts/s fwd+adjoint", "value": shots * npts * nt / (ms_ * 1e-3) / 1e9, "unit": "Gpts/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"rho_l2_gradient_{BN_NZI}x{BN_NXI}_habc{BN_W}_o2_nt{nt}_{shots}shots",
                       "grid": [nz, nx], "shots": shots, "nt": nt, "ckpt_every": ck,
                       "l2": "inputs larger than L2 (70 MB per field)"},
            "shots_per_s": shots / (ms_ * 1e-3), "phases_ms": {"forward": fwd_ms, "adjoint": rev_ms},
            "roofline": {"kernel": "habc_bwd_tile_kernel (variable density, far + near tiles)", "bound": "hbm", "achieved": rev_gbs,
                         "peak": peak, "peak_kind": kind, "unit": "GB/s", "frac": rev_gbs / peak, "traffic": None,
                         "bytes_per_launch": rev_bytes, "launch_ms": rev_ms / (nt - 1)},
            "roofline_forward": {"kernel": "acoustic_fwd_tile_kernel<HABC> (variable density)", "achieved": fwd_gbs,
                                 "frac": fwd_gbs / peak, "unit": "GB/s", "launch_ms": fwd_ms / nt},
            # per step: NT forward, 2 (NT-1) reverse (far and near tiles), share planes, coefficients,
            # misfit, 5 reductions
            "gpu_launches": args.steps * (nt + 2 * (nt - 1) + 8), "clocks": clocks.summary()}
    if not args.no_e2e:
        line["e2e"] = e2e_models(args, dev, "acoustic_rho_habc", "habc", BN_W, BN_DT, BN_H, 2,
                                 dict(zip(("vp", "rho"), init)), ("vp", "rho"), obs.cpu(), 1, wav, src, rec, nt,
                                 ["h1"], ["h1"])
    print(json.dumps(line))
    return 0


# -------------------------------------------------------- uneven batch ---
# 4 grid sizes (interior 200x400, 300x700, 400x1000, 600x1500 + 50-cell PML),
# 64 shots each, trace lengths 1500 / 2000 / 3000 / 4000 steps, 8th order,
# smooth random vp 1500-4500 m/s (seeded), forward with records on row 2.
UNEVEN = [(200, 400, 1500), (300, 700, 2000), (400, 1000, 3000), (600, 1500, 4000)]


def bench_uneven(args):
    import torch
    from scipy.ndimage import gaussian_filter
    from seistorch_gb300 import _native, engine, tuning
    from seistorch_gb300.pml import generate_pml_coefficients_2d
    from seistorch_gb300.utils import ricker_wave
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is timed on the acoustic "
                          "gradient workload only"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    shots = args.shots if args.shots != NSHOTS else 64
    scale = 1.0 if args.nt == NT else args.nt / 4000.0
    rng = np.random.default_rng(0)
    groups = []
    for nzi, nxi, nt in UNEVEN:
        nt = max(8, int(nt * scale))
        noise = gaussian_filter(rng.standard_normal((nzi, nxi)), sigma=20)
        vp = 1500.0 + 3000.0 * (noise - noise.min()) / (noise.max() - noise.min())
        vp = np.pad(vp, WIDTH, mode="edge")
        nz, nx = vp.shape
        d = generate_pml_coefficients_2d((nz, nx), WIDTH).to(device=dev, dtype=torch.float32)
        xs = np.linspace(0, nxi - 1, shots).round().astype(int)
        src = [[(WIDTH + 2, WIDTH + int(x))] for x in xs]
        rec = [([WIDTH + 2] * nxi, list(range(WIDTH, WIDTH + nxi)))] * shots
        wav = ricker_wave(FM, DT, nt, delay=int(1.2 / FM / DT), dtype="numpy")
        prop = engine.AcousticPropagator(nz, nx, DT, H, ORDER, "pml", WIDTH, False, dev)
        acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
        groups.append((prop, torch.tensor(vp, dtype=torch.float32, device=dev), d, acq))
    # autotuner: per-grid winners, then the batch timed on each of them
    per_grid = [tuning.tune_grid(p.nz, p.nx, shots, ORDER, DT, H, WIDTH, dev, steps=24, adjoint=False)[0][0]
                for p, _, _, _ in groups]
    batch = engine.UnevenBatch(groups)
    best, tune_ms = tuning.tune_batch(batch.run, per_grid)
    batch.plan()
    pts = batch.points()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        batch.replay()
    torch.cuda.synchronize()
    with ClockSampler(0) as clocks:
        t0, t1 = ev(), ev()
        t0.record(stream)
        for _ in range(args.steps):
            batch.replay()
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    # same grids one after another, one loop each (no graph), for reference
    t2, t3 = ev(), ev()
    t2.record(stream)
    for prop, vp, d, acq in groups:
        prop.forward(vp, d, acq)
    t3.record(stream)
    torch.cuda.synchronize()
    seq_ms = t2.elapsed_time(t3)
    npts_step = sum(acq.nshots * p.nz * p.nx for p, _, _, acq in groups)
    peak, kind = measured_peaks()
    gbs = pts * BYTES_FWD / (ms * 1e-3) / 1e9
    line = {"metric": "Gpts/s fwd (uneven batch)", "value": pts / (ms * 1e-3) / 1e9, "unit": "Gpts/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "uneven_forward_4grids_x%dshots" % shots,
                       "grids": [[p.nz, p.nx, acq.nt] for p, _, _, acq in groups], "shots_per_grid": shots,
                       "order": ORDER, "launch": "one persistent launch per step, whole loop one CUDA graph",
                       "variant_per_grid": per_grid, "variant_batch": best,
                       "l2": "inputs larger than L2"},
            "shots_per_s": len(groups) * shots / (ms * 1e-3),
            "sequential_loops_ms": seq_ms, "tuning_ms": tune_ms,
            "roofline": {"kernel": "acoustic_fwd_batch_kernel", "bound": "hbm", "achieved": gbs, "peak": peak,
                         "peak_kind": kind, "unit": "GB/s", "frac": gbs / peak, "traffic": None,
                         "bytes_per_point": BYTES_FWD, "points_per_step_max": npts_step},
            "gpu_launches": args.steps * max(acq.nt for _, _, _, acq in groups), "clocks": clocks.summary()}
    batch.close()
    print(json.dumps(line))
    return 0


# ---------------------------------------------------- learned FWI (C5) ---
# Network: 4-level U-Net, 32 base channels (~1.16 M parameters), bf16
# weights / fp32 accumulation on tcgen05, inputs raw gradient +
# illumination on 256 x 512.  Pairs: seeded random layered + anomaly models
# (1500-4500 m/s), gradient at the smoothed model from 8 shots x 1500 steps.
# FWI: 20 iterations, 32 shots, 3000 steps, 8 Hz, on a held-out model;
# plain illumination-preconditioned gradient vs the learned update (misfit-
# judged, plain fallback).  value = wall time for the learned run to reach
# the plain run's final misfit / the plain run's wall time.


def conv_flops(B, H, W):
    """FLOPs of one forward pass of the network (multiply-add = 2)."""
    from seistorch_gb300.learned import LAYERS
    res = {"e1a": 0, "e1b": 0, "e2a": 1, "e2b": 1, "e3a": 2, "e3b": 2, "b4": 3, "d3": 2, "d2": 1, "d1": 0,
           "out": 0}
    return sum(2.0 * B * (H >> res[n]) * (W >> res[n]) * ci * co * 9 for n, ci, co, _ in LAYERS)


def bench_net(args):
    """Tensor-core throughput of the preconditioner network alone: forward and
    one training step (forward + backward + Adam) on a batch of 8 random
    2 x 256 x 512 inputs."""
    import torch
    from seistorch_gb300 import _native
    from seistorch_gb300.learned import PrecondNet
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    torch.manual_seed(0)
    x = torch.randn(8, 2, 256, 512, device=dev)
    y = torch.randn(8, 256, 512, device=dev) * 0.1
    net = PrecondNet(dev, seed=0)
    for _ in range(args.warmup):
        net.train_batch(x, y, 1e-4)
    torch.cuda.synchronize()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    a, b, c = ev(), ev(), ev()
    a.record()
    for _ in range(args.steps):
        net.forward(x)
    b.record()
    for _ in range(args.steps):
        net.train_batch(x, y, 1e-4)
    c.record()
    torch.cuda.synchronize()
    fwd = a.elapsed_time(b) / args.steps
    step = b.elapsed_time(c) / args.steps
    fl = conv_flops(8, 256, 512)
    peak = None
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            peak = json.load(f).get("bf16_tflops")
    t_f = fl / (fwd * 1e-3) / 1e12
    print(json.dumps({"metric": "network TFLOP/s (forward)", "value": t_f, "unit": "TFLOP/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "bf16/fp32acc",
                      "data": "synthetic", "config": {"workload": "precond_unet_b8_256x512"},
                      "forward_ms": fwd, "train_step_ms": step, "train_tflops": 3 * fl / (step * 1e-3) / 1e12,
                      "roofline": {"bound": "tensor", "achieved": t_f, "peak": peak, "unit": "TFLOP/s",
                                   "frac": t_f / peak if peak else None}}))
    return 0


def bench_learned(args):
    import torch
    from seistorch_gb300 import _native, fwi
    from seistorch_gb300.learned import PrecondNet, n_params
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned preconditioner; its "
                          "arm is timed on the acoustic gradient workload"}))
        return 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _native.load(build_if_missing=False)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    # pairs on the inversion's own survey (32 shots, 3000 steps, 8 Hz)
    train_sv = fwi.Survey(256, 512, shots=32, nt=3000, fm=8.0, device=dev)
    X, Y = fwi.make_pairs(args.pairs, train_sv, seed=0, log=log)
    torch.cuda.synchronize()
    t_pairs = time.perf_counter() - t0
    net = PrecondNet(dev, seed=0)
    # tensor-core throughput of the network (forward + backward, batch 8)
    xb, yb = X[:8].contiguous(), Y[:8].contiguous()
    for _ in range(3):
        net.train_batch(xb, yb, 0.0)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    e0, e1 = ev(), ev()
    e0.record()
    for _ in range(10):
        net.forward(xb)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / 10
    net = PrecondNet(dev, seed=0)
    t1 = time.perf_counter()
    hist = fwi.train(net, X, Y, epochs=args.epochs, batch=8, lr=1e-3, log=log)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    if args.save_net:
        np.savez(args.save_net, **net.state_dict())
    # held-out inversion
    sv = train_sv
    rng = np.random.default_rng(12345)
    vt = fwi.random_model(rng, 256, 512)
    v0 = fwi.smooth(vt)
    obs = sv.records(sv.pad(vt))
    plain = fwi.invert(sv, obs, v0, iters=args.iters, log=lambda m: log("plain " + m))
    learned = fwi.invert(sv, obs, v0, iters=args.iters, net=net, log=lambda m: log("learned " + m))
    target = plain["misfit"][-1]
    t_plain = plain["time"][-1]
    reach = next((t for m, t in zip(learned["misfit"], learned["time"]) if m <= target), None)
    ratio = reach / t_plain if reach is not None else None
    # model error relative to the starting model's (1 = no better than the start)
    model_err = lambda r: float(torch.linalg.norm(r["model"] - torch.as_tensor(vt, device=dev, dtype=torch.float32))
                                / np.linalg.norm(vt - v0))
    peak = None
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            peak = json.load(f).get("bf16_tflops")
    tflops = conv_flops(8, 256, 512) / (fwd_ms * 1e-3) / 1e12
    line = {"metric": "FWI time-to-misfit, learned vs plain", "value": ratio, "unit": "x plain wall time",
            "higher_is_better": False, "n_gpus": 1, "steps": 1, "warmup": 0, "vs_baseline": None,
            "dtype": "bf16 weights / fp32 accumulate (network), f32 (solver)", "data": "synthetic",
            "config": {"workload": "learned_preconditioner_fwi_256x512_32shots_nt3000", "pairs": args.pairs,
                       "pair_survey": "the inversion's: 32 shots x 3000 steps, 8 Hz",
                       "start": f"true model Gaussian-smoothed, sigma {fwi.START_SIGMA:g} cells",
                       "plain_method": "illumination-preconditioned PR conjugate gradient + parabolic line search",
                       "epochs": args.epochs, "iters": args.iters,
                       "params": n_params()},
            "plain": {"final_misfit": target, "wall_s": t_plain, "misfit": plain["misfit"],
                      "time": plain["time"], "model_error": model_err(plain)},
            "learned": {"misfit": learned["misfit"], "time": learned["time"], "learned_steps": learned["learned_steps"],
                        "reach_s": reach, "model_error": model_err(learned)},
            "training": {"pairs_s": t_pairs, "train_s": t_train, "loss": hist},
            "roofline": {"kernel": "nn_gemm_kernel (network forward, batch 8, 256x512)", "bound": "tensor",
                         "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": (tflops / peak) if peak else None, "forward_ms": fwd_ms}}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
