"""GPU parity of the elastic velocity-stress kernels against the reference's
own outputs (golden vectors) and the CPU oracle.

Tolerances (relative L2): records and final fields vs the reference in fp64
and fp32 <= 1e-5; single step vs the fp64 oracle <= 2e-6; gradients inside
the undamped box vs the reference's autograd gradient <= 1e-4.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint, fd2d
from tests.golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ["vx", "vz", "txx", "tzz", "txz"]


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _run(g, dev, requires_grad=False, ckpt=0):
    from seistorch_gb300 import elastic_engine, engine
    nz, nx = g["models"]["vp"].shape
    prop = elastic_engine.ElasticPropagator(nz, nx, g["dt"], g["h"], g["width"], g["multiple"], dev)
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=requires_grad)
    vp, vs, rho = t(g["models"]["vp"]), t(g["models"]["vs"]), t(g["models"]["rho"])
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    io, nch = elastic_engine.make_io(g["source_type"], g["receiver_type"])
    rec, _ = elastic_engine.elastic_records(vp, vs, rho, prop, d, acq, io, nch, False, ckpt)
    B = len(g["sources"])
    nrec = len(g["receivers"][0][0])
    per_shot = rec.reshape(g["nt"], B, nrec, nch).permute(1, 0, 2, 3)
    return (vp, vs, rho), per_shot, prop


def test_forward_through_wavernn(dev):
    """The user path for the elastic equation: build_model(dict config) ->
    WaveRNN -> per-shot records (nt, nrec, vx / vz), against the reference."""
    from seistorch_gb300 import build_model
    g = load("elastic")
    w = g["width"]
    models = {k: g["models"][k][w:-w, w:-w] for k in ("vp", "vs", "rho")}
    cfg = {"equation": "elastic", "dtype": "float32",
           "geom": {"dt": g["dt"], "h": g["h"], "nt": g["nt"], "boundary": {"type": "pml", "width": w},
                    "multiple": False, "boundary_saving": True, "source_type": list(g["source_type"]),
                    "receiver_type": list(g["receiver_type"]), "spatial_order": 2,
                    "invlist": {"vp": False, "vs": False, "rho": False}}}
    _, model = build_model(cfg, device=dev, mode="forward", models=models)
    srcs = [[int(x) - w, int(z) - w] for z, x in g["src"]]
    recs = [[[int(x) - w for x in xs], [int(z) - w for z in zs]] for zs, xs in g["receivers"]]
    model.reset_geom(list(range(len(srcs))), srcs, recs, cfg)
    y = model(torch.tensor(g["wavelet"])[None])
    got = np.stack([t.detach().cpu().numpy() for t in y])
    assert got.shape == g["records"].shape
    assert rel_l2(got, g["records"]) < 1e-5


@pytest.mark.parametrize("name", ["elastic", "elastic_multiple"])
def test_forward_matches_reference(dev, name):
    from seistorch_gb300 import elastic_engine, engine
    g = load(name)
    _, rec, _ = _run(g, dev)
    got = rec.cpu().numpy()
    assert got.shape == g["records"].shape
    assert rel_l2(got, g["records"]) < 1e-5
    assert rel_l2(got, g["records_f32"]) < 1e-5
    # final wavefields of shot 0
    nz, nx = g["models"]["vp"].shape
    prop = elastic_engine.ElasticPropagator(nz, nx, g["dt"], g["h"], g["width"], g["multiple"], dev)
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    io, nch = elastic_engine.make_io(g["source_type"], g["receiver_type"])
    _, state, _ = prop.forward(t(g["models"]["vp"]), t(g["models"]["vs"]), t(g["models"]["rho"]), t(g["d"]),
                               acq, io, nch)
    for f, field in zip(FIELDS, prop.final_fields(state)):
        assert rel_l2(field[0].cpu().numpy(), g["field_" + f]) < 1e-5, f


def test_single_step_matches_oracle(dev):
    from seistorch_gb300.equations2d import elastic
    g = load("elastic")
    rng = np.random.default_rng(0)
    nz, nx = g["models"]["vp"].shape
    fields = [rng.standard_normal((3, nz, nx)).astype(np.float32) for _ in range(5)]
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    out = elastic._time_step(t(g["models"]["vp"]), t(g["models"]["vs"]), t(g["models"]["rho"]),
                             *[t(f) for f in fields], torch.tensor(g["dt"]), torch.tensor(g["h"]), t(g["d"]))
    want = fd2d.elastic_step(g["models"]["vp"], g["models"]["vs"], g["models"]["rho"], *fields, g["dt"], g["h"],
                             g["d"])
    for f, a, b in zip(FIELDS, out, want):
        assert rel_l2(a.cpu().numpy(), b) < 2e-6, f


def _torch_step(vp, vs, rho, fields, dt, h, d):
    """The step of elastic.py:7-37 in plain torch (float64 reference)."""
    def fwd(x, dim):  # x[i] - x[i-1], 0 at i = 0
        y = x - torch.roll(x, 1, dim)
        y.select(dim, 0).zero_()
        return y

    def bwd(x, dim):  # x[i+1] - x[i], 0 at the last index
        y = torch.roll(x, -1, dim) - x
        y.select(dim, -1).zero_()
        return y
    vx, vz, txx, tzz, txz = fields
    lam, mu = rho * (vp ** 2 - 2 * vs ** 2), rho * vs ** 2
    c = 0.5 * dt * d
    sxx = (dt / h * ((lam + 2 * mu) * fwd(vx, 2) + lam * bwd(vz, 1)) + (1 - c) * txx) / (1 + c)
    szz = (dt / h * ((lam + 2 * mu) * bwd(vz, 1) + lam * fwd(vx, 2)) + (1 - c) * tzz) / (1 + c)
    sxz = (dt * mu / h * (bwd(vz, 2) + fwd(vx, 1)) + (1 - c) * txz) / (1 + c)
    nvx = (dt / (rho * h) * (bwd(sxx, 2) + bwd(sxz, 1)) + (1 - c) * vx) / (1 + c)
    nvz = (dt / (rho * h) * (fwd(sxz, 2) + fwd(szz, 1)) + (1 - c) * vz) / (1 + c)
    return nvx, nvz, sxx, szz, sxz


def test_single_step_vjp_matches_torch_autograd(dev):
    """Autograd through one native step vs torch autograd of the same step in
    float64."""
    from seistorch_gb300.equations2d import elastic
    g = load("elastic")
    rng = np.random.default_rng(1)
    nz, nx = g["models"]["vp"].shape
    fields = [rng.standard_normal((2, nz, nx)) for _ in range(5)]
    gouts = [rng.standard_normal((2, nz, nx)) for _ in range(5)]
    mods = [g["models"][n] for n in ("vp", "vs", "rho")]
    t32 = lambda a, rg=False: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=rg)
    m32 = [t32(m, True) for m in mods]
    f32 = [t32(f, True) for f in fields]
    out = elastic._time_step(*m32, *f32, torch.tensor(g["dt"]), torch.tensor(g["h"]), t32(g["d"]))
    sum((o * t32(go)).sum() for o, go in zip(out, gouts)).backward()
    t64 = lambda a: torch.tensor(a, dtype=torch.float64, requires_grad=True)
    m64 = [t64(m) for m in mods]
    f64 = [t64(f) for f in fields]
    out64 = _torch_step(*m64, f64, g["dt"], g["h"], torch.tensor(g["d"]))
    sum((o * torch.tensor(go)).sum() for o, go in zip(out64, gouts)).backward()
    for name, a, b in zip(FIELDS, f32, f64):
        assert rel_l2(a.grad.cpu().numpy(), b.grad.numpy()) < 1e-5, name
    for name, a, b in zip(("vp", "vs", "rho"), m32, m64):
        assert rel_l2(a.grad.cpu().numpy(), b.grad.numpy()) < 1e-5, name


@pytest.mark.parametrize("ckpt", [0, 25])
def test_bs_gradient_matches_reference_autograd(dev, ckpt):
    """L2 misfit against zero data: the fused boundary-saving elastic adjoint
    vs the reference's autograd gradient, inside the undamped box."""
    g = load("grad_elastic_zeroobs")
    (vp, vs, rho), rec, _ = _run(g, dev, requires_grad=True, ckpt=ckpt)
    loss = (rec ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    w = g["width"]
    box = (slice(w, -w), slice(w, -w))
    for name, p in (("vp", vp), ("vs", vs), ("rho", rho)):
        got = p.grad.cpu().numpy()
        assert rel_l2(got[box], g["grad_" + name][box]) < 1e-4, name
        mask = np.ones_like(got, bool)
        mask[box] = False
        assert np.all(got[mask] == 0), name


def test_bs_gradient_matches_oracle_adjoint_same_residual(dev):
    """With observed data: drive the exact fp64 adjoint with the GPU's own
    residual (the residual amplifies fp32 forward rounding)."""
    g = load("grad_elastic")
    (vp, vs, rho), rec, _ = _run(g, dev, requires_grad=True, ckpt=30)
    obs = torch.tensor(g["obs"], dtype=torch.float32, device=dev)
    ((rec - obs) ** 2).sum().backward()
    resid = 2.0 * (rec.detach().cpu().double().numpy() - g["obs"])
    want = adjoint.elastic_gradient(g["models"]["vp"], g["models"]["vs"], g["models"]["rho"], g["d"], g["dt"],
                                    g["h"], g["wavelet"], g["sources"], g["receivers"], list(resid),
                                    source_type=tuple(g["source_type"]), receiver_type=tuple(g["receiver_type"]))
    w = g["width"]
    box = (slice(w, -w), slice(w, -w))
    for k, (name, p) in enumerate((("vp", vp), ("vs", vs), ("rho", rho))):
        assert rel_l2(p.grad.cpu().numpy()[box], want[k][box]) < 1e-4, name


def test_forward_config3_shape_vs_fp64_oracle(dev):
    """Elastic config shapes (300x800 + 50-cell PML, dx = 5 m, dt = 0.5 ms,
    explosive source, vx/vz receivers on every cell), 1000 steps, one shot:
    GPU fp32 records vs the fp64 oracle within 1e-5."""
    from seistorch_gb300 import elastic_engine, engine
    nzi, nxi, w = 300, 800, 50
    zz, xx = np.mgrid[0:nzi, 0:nxi]
    vpi = np.where(zz < 100, 2000.0, np.where(zz < 200 + (xx > 400) * 20, 3500.0, 5000.0))
    vp = fd2d.pad_model(vpi, w)
    vs = vp / 1.73
    rho = 310.0 * vp ** 0.25
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    nt, dt, h = 1000, 0.0005, 5.0
    wav = fd2d.ricker(12.0, dt, nt, delay=int(1.2 / 12.0 / dt))
    src = [[(w + 2, w + 400)]]
    rec = [([w + 2] * nxi, list(range(w, w + nxi)))]
    want = fd2d.forward("elastic", {"vp": vp, "vs": vs, "rho": rho}, d, dt, h, wav, src, rec)["records"][0]
    prop = elastic_engine.ElasticPropagator(nz, nx, dt, h, w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    io, nch = elastic_engine.make_io(["txx", "tzz"], ["vx", "vz"])
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    r, _ = elastic_engine.elastic_records(t(vp), t(vs), t(rho), prop, t(d), acq, io, nch)
    err = rel_l2(r.cpu().numpy().reshape(nt, nxi, 2), want)
    print(f"elastic config-3 shape records rel L2 vs fp64 oracle: {err:.3e}")
    assert err < 1e-5
