"""GPU parity of the acoustic kernels against the reference's own outputs
(golden vectors) and the CPU oracle.

Tolerances (relative L2): records vs the reference in fp64 <= 1e-5; vs the
reference's fp32 run <= 1e-5 (both are fp32 paths; over these short runs the
two fp32 rounding histories stay within it); gradients inside the undamped
box vs the reference's autograd gradient <= 1e-4.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint, fd2d
from tests.golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu

ACOUSTIC_CASES = ["acoustic_pml_o2", "acoustic_pml_o4", "acoustic_pml_o8", "acoustic_pml_o4_multiple",
                  "acoustic_habc_o2", "acoustic_habc_o4", "acoustic_habc_o2_multiple"]


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _prop(g, dev):
    from seistorch_gb300 import engine
    nz, nx = g["models"]["vp"].shape
    return engine.AcousticPropagator(nz, nx, g["dt"], g["h"], g["order"], "habc" if g["habc"] else "pml",
                                     g["width"], g["multiple"], dev)


def _forward(g, dev, requires_grad=False, ckpt=0):
    from seistorch_gb300 import engine
    nz, nx = g["models"]["vp"].shape
    prop = _prop(g, dev)
    vp = torch.tensor(g["models"]["vp"], dtype=torch.float32, device=dev, requires_grad=requires_grad)
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    rec, _ = engine.acoustic_loop(vp, prop, d, acq, False, ckpt)
    B = len(g["sources"])
    nrec = len(g["receivers"][0][0])
    per_shot = rec.reshape(g["nt"], B, nrec, 1).permute(1, 0, 2, 3)
    return vp, rec, per_shot


@pytest.mark.parametrize("name", ACOUSTIC_CASES)
def test_forward_matches_reference(dev, name):
    g = load(name)
    _, _, rec = _forward(g, dev)
    got = rec.detach().cpu().numpy()
    assert got.shape == g["records"].shape
    assert rel_l2(got, g["records"]) < 1e-5
    assert rel_l2(got, g["records_f32"]) < 1e-5


def test_forward_through_wavernn(dev):
    """The user path: build_model(dict config) -> WaveRNN -> TensorList."""
    from seistorch_gb300 import build_model
    from seistorch_gb300.acquisition import setup_acquisition  # noqa: F401
    g = load("acoustic_pml_o4")
    w = g["width"]
    vp_int = g["models"]["vp"][w:-w, w:-w]
    cfg = {"equation": "acoustic", "dtype": "float32",
           "geom": {"dt": g["dt"], "h": g["h"], "nt": g["nt"], "boundary": {"type": "pml", "width": w},
                    "multiple": False, "boundary_saving": True, "source_type": ["h1"],
                    "receiver_type": ["h1"], "spatial_order": 4, "invlist": {"vp": False}}}
    _, model = build_model(cfg, device=dev, mode="forward", models={"vp": vp_int})
    srcs = [[int(x) - w, int(z) - w] for z, x in g["src"]]
    recs = [[[int(x) - w for x in xs], [int(z) - w for z in zs]] for zs, xs in g["receivers"]]
    model.reset_geom([0, 1], srcs, recs, cfg)
    y = model(torch.tensor(g["wavelet"])[None])
    got = np.stack([t.detach().cpu().numpy() for t in y])
    assert rel_l2(got, g["records"]) < 1e-5


def test_wavernn_acquisition_cache_follows_the_geometry(dev):
    """WaveRNN keeps the batch's source / receiver tables between calls: a
    second call with a doubled wavelet doubles the records (the cached tables
    with the new wavelet), reset_geom with the shots in reverse order gives
    the reference's records in reverse order, and an in-place shift of the
    receiver coordinates changes them (the cache key follows the buffers)."""
    from seistorch_gb300 import build_model
    g = load("acoustic_pml_o4")
    w = g["width"]
    vp_int = g["models"]["vp"][w:-w, w:-w]
    cfg = {"equation": "acoustic", "dtype": "float32",
           "geom": {"dt": g["dt"], "h": g["h"], "nt": g["nt"], "boundary": {"type": "pml", "width": w},
                    "multiple": False, "boundary_saving": True, "source_type": ["h1"],
                    "receiver_type": ["h1"], "spatial_order": 4, "invlist": {"vp": False}}}
    _, model = build_model(cfg, device=dev, mode="forward", models={"vp": vp_int})
    srcs = [[int(x) - w, int(z) - w] for z, x in g["src"]]
    recs = [[[int(x) - w for x in xs], [int(z) - w for z in zs]] for zs, xs in g["receivers"]]
    wav = torch.tensor(g["wavelet"])[None]
    records = lambda y: np.stack([t.detach().cpu().numpy() for t in y])
    model.reset_geom([0, 1], srcs, recs, cfg)
    first = records(model(wav))
    twice = records(model(2.0 * wav))
    assert rel_l2(first, g["records"]) < 1e-5
    assert rel_l2(twice, 2.0 * first) < 1e-6
    model.reset_geom([0, 1], srcs[::-1], recs[::-1], cfg)
    assert rel_l2(records(model(wav)), g["records"][::-1]) < 1e-5
    with torch.no_grad():
        for probe in model.probes:
            for name, buf in probe.named_buffers():
                if name == "y":
                    buf.add_(1)  # every receiver one row deeper
    moved = records(model(wav))
    assert rel_l2(moved, g["records"][::-1]) > 1e-3


@pytest.mark.parametrize("name", ["acoustic_pml_o2", "acoustic_pml_o4", "acoustic_habc_o2"])
def test_single_step_matches_oracle(dev, name):
    from seistorch_gb300.equations2d import acoustic, acoustic_habc
    g = load(name)
    mod = acoustic_habc if g["habc"] else acoustic
    mod.spatial_order = g["order"]
    rng = np.random.default_rng(0)
    nz, nx = g["models"]["vp"].shape
    h1 = rng.standard_normal((3, nz, nx)).astype(np.float32)
    h2 = rng.standard_normal((3, nz, nx)).astype(np.float32)
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    y, h1o = mod._time_step(t(g["models"]["vp"]), t(h1), t(h2), torch.tensor(g["dt"]), torch.tensor(g["h"]),
                            t(g["d"]))
    if g["habc"]:
        want, _ = fd2d.acoustic_habc_step(g["models"]["vp"], h1, h2, g["dt"], g["h"], g["d"], g["order"])
    else:
        want, _ = fd2d.acoustic_step(g["models"]["vp"], h1, h2, g["dt"], g["h"], g["d"], g["order"])
    assert rel_l2(y.cpu().numpy(), want) < 2e-6
    assert torch.equal(h1o.cpu(), torch.tensor(h1))
    mod.spatial_order = 2


def test_single_step_vjp_matches_oracle(dev):
    """Autograd through one native step equals the exact transposed step."""
    from seistorch_gb300.equations2d import acoustic
    g = load("acoustic_pml_o4")
    acoustic.spatial_order = 4
    rng = np.random.default_rng(1)
    nz, nx = g["models"]["vp"].shape
    vp0 = g["models"]["vp"]
    h1 = rng.standard_normal((2, nz, nx))
    h2 = rng.standard_normal((2, nz, nx))
    gy = rng.standard_normal((2, nz, nx))
    t = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    vp, a1, a2 = t(vp0, True), t(h1, True), t(h2, True)
    y, _ = acoustic._time_step(vp, a1, a2, torch.tensor(g["dt"]), torch.tensor(g["h"]), t(g["d"]))
    (y * t(gy)).sum().backward()
    # exact VJP in float64: y = A h1 - Bc h2 + Kv Lh(h1)
    d, dt, h = g["d"], g["dt"], g["h"]
    inv = 1 / (dt ** -2 + d / dt)
    A, Bc, Kv = 2 * inv / dt ** 2, inv * (dt ** -2 - d / dt), inv * vp0 ** 2
    w_h1 = A * gy + fd2d.laplacian(Kv * gy, 4, h)
    w_h2 = -Bc * gy
    w_vp = np.sum(gy * fd2d.laplacian(h1, 4, h), 0) * 2 * vp0 * inv
    assert rel_l2(a1.grad.cpu().numpy(), w_h1) < 1e-5
    assert rel_l2(a2.grad.cpu().numpy(), w_h2) < 1e-6
    assert rel_l2(vp.grad.cpu().numpy(), w_vp) < 1e-5
    acoustic.spatial_order = 2


@pytest.mark.parametrize("name", ["grad_acoustic_pml_o4_zeroobs", "grad_acoustic_pml_o8_zeroobs"])
@pytest.mark.parametrize("ckpt", [0, 25])
def test_bs_gradient_matches_reference_autograd(dev, name, ckpt):
    """L2 misfit against zero data (a residual without cancellation): the
    fused boundary-saving adjoint vs the reference's autograd gradient."""
    g = load(name)
    vp, rec, per_shot = _forward(g, dev, requires_grad=True, ckpt=ckpt)
    loss = (per_shot ** 2).sum()
    loss.backward()
    w = g["width"]
    box = (slice(w, -w), slice(w, -w))
    got = vp.grad.cpu().numpy()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    assert rel_l2(got[box], g["grad_vp"][box]) < 1e-4
    # outside the undamped box the boundary-saving gradient is defined as 0
    mask = np.ones_like(got, bool)
    mask[box] = False
    assert np.all(got[mask] == 0)


@pytest.mark.parametrize("name", ["grad_acoustic_pml_o4", "grad_acoustic_pml_o8"])
def test_bs_gradient_matches_oracle_adjoint_same_residual(dev, name):
    """With observed data the residual syn - obs is a small difference of two
    similar runs, so fp32 forward rounding is amplified in it; drive the
    exact fp64 adjoint with the GPU's own residual to test the adjoint."""
    g = load(name)
    vp, rec, per_shot = _forward(g, dev, requires_grad=True, ckpt=30)
    obs = torch.tensor(g["obs"], dtype=torch.float32, device=dev)
    ((per_shot - obs) ** 2).sum().backward()
    resid = 2.0 * (per_shot.detach().cpu().double().numpy() - g["obs"])
    want = adjoint.acoustic_pml_gradient(g["models"]["vp"], g["d"], g["dt"], g["h"], g["wavelet"],
                                         g["sources"], g["receivers"], list(resid), order=g["order"])
    w = g["width"]
    box = (slice(w, -w), slice(w, -w))
    assert rel_l2(vp.grad.cpu().numpy()[box], want[box]) < 1e-4


def test_forward_config1_size_vs_fp64_oracle(dev):
    """Config-1 shapes (128x256 + 50-cell PML, 4th order, 1000 steps): GPU fp32
    records vs the fp64 oracle within 1e-5 (the reference's own fp32 path
    is about 2.5e-5 off here)."""
    from seistorch_gb300 import engine
    nzi, nxi, w = 128, 256, 50
    vpi = np.zeros((nzi, nxi))
    vpi[:43], vpi[43:86], vpi[86:] = 1500.0, 2500.0, 3500.0
    zz, xx = np.mgrid[0:nzi, 0:nxi]
    vpi += 300 * np.exp(-((zz - 64) ** 2 + (xx - 128) ** 2) / (2 * 10 ** 2))
    vp = fd2d.pad_model(vpi, w)
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    nt = 1000
    wav = fd2d.ricker(10.0, 0.001, nt, delay=100)
    shots = [0, 4]
    src = [[(w + 2, w + 16 + 32 * k)] for k in shots]
    rec = [([w + 2] * nxi, list(range(w, w + nxi)))] * len(shots)
    want = np.stack(fd2d.forward("acoustic", {"vp": vp}, d, 0.001, 10.0, wav, src, rec, order=4)["records"])
    prop = engine.AcousticPropagator(nz, nx, 0.001, 10.0, 4, "pml", w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    r, _ = engine.acoustic_loop(torch.tensor(vp, dtype=torch.float32, device=dev), prop,
                                torch.tensor(d, dtype=torch.float32, device=dev), acq)
    got = r.cpu().numpy().reshape(nt, len(shots), nxi, 1).transpose(1, 0, 2, 3)
    err = rel_l2(got, want)
    print(f"config-1 records rel L2 vs fp64 oracle: {err:.3e}")
    assert err < 1e-5


@pytest.mark.parametrize("name", ["grad_acoustic_habc_o2_zeroobs", "grad_acoustic_habc_o4_zeroobs",
                                  "grad_acoustic_habc_o2_multiple_zeroobs"])
@pytest.mark.parametrize("ckpt", [0, 25])
def test_habc_gradient_matches_reference_autograd(dev, name, ckpt):
    """HABC (acoustic_habc.py): the boundary-saving adjoint with the exact
    transposed one-way blend vs the reference's autograd gradient, inside
    the undamped box (rows from 0 with ``multiple``); 0 outside."""
    g = load(name)
    vp, rec, per_shot = _forward(g, dev, requires_grad=True, ckpt=ckpt)
    loss = (per_shot ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    w = g["width"]
    box = (slice(0 if g["multiple"] else w, -w), slice(w, -w))
    got = vp.grad.cpu().numpy()
    assert rel_l2(got[box], g["grad_vp"][box]) < 1e-4
    mask = np.ones_like(got, bool)
    mask[box] = False
    assert np.all(got[mask] == 0)


def test_every_forward_variant_gives_the_same_records(dev):
    """All compiled tile-pipeline variants (rows per tile, warps, stages,
    previous field via TMA) compute the same arithmetic: identical records,
    within 1e-5 of the reference."""
    from seistorch_gb300 import tuning
    g = load("acoustic_pml_o8")
    outs = []
    try:
        for cfg in range(len(tuning.FWD_VARIANTS)):
            tuning.select(cfg, 0)
            _, _, rec = _forward(g, dev)
            outs.append(rec.detach().cpu().numpy())
    finally:
        tuning.select(*tuning.DEFAULT)
    for o in outs:
        assert np.array_equal(o, outs[0])
    assert rel_l2(outs[0], g["records"]) < 1e-5


@pytest.mark.parametrize("name", ["grad_acoustic_pml_o4_zeroobs", "grad_acoustic_pml_o8_zeroobs"])
def test_every_adjoint_variant_gives_the_same_gradient(dev, name):
    """All compiled adjoint variants (rows per tile, warps, stages, point
    rows and coefficient rows through the TMA stage) compute the same
    arithmetic: gradients equal up to the order of the reduction atomics
    (relative L2 <= 1e-6 between variants), each within 1e-4 of the
    reference's autograd gradient, with checkpoints every 25 steps."""
    from seistorch_gb300 import tuning
    g = load(name)
    w = g["width"]
    box = (slice(w, -w), slice(w, -w))
    grads = []
    try:
        for cfg in range(len(tuning.BWD_VARIANTS)):
            tuning.select(tuning.DEFAULT[0], cfg)
            vp, _, per_shot = _forward(g, dev, requires_grad=True, ckpt=25)
            (per_shot ** 2).sum().backward()
            grads.append(vp.grad.cpu().numpy())
    finally:
        tuning.select(*tuning.DEFAULT)
    for cfg, got in enumerate(grads):
        assert rel_l2(got, grads[0]) < 1e-6, cfg
        assert rel_l2(got[box], g["grad_vp"][box]) < 1e-4, cfg
