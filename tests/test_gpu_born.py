"""GPU parity of Born modelling (acoustic_lsrtm_habc: background field with
the sources, scattered field driven by m vp^2 dt^2 lap(p), both under the
HABC blend, receivers on the scattered field) against the reference's own
outputs (golden vectors made by tests/golden/make_golden.py) and the fp64
oracle.

Tolerances (relative L2): scattered-field records vs the reference in fp64
<= 1e-5; dJ/dm inside the undamped box vs the reference's autograd gradient
<= 1e-4, and 0 outside it.
"""
import numpy as np
import pytest
import torch

from oracle import fd2d
from tests.golden_cases import BORN_GRAD_CASES, load, rel_l2

pytestmark = pytest.mark.gpu

BORN_CASES = ["born_habc_o2", "born_habc_o4", "born_habc_o2_multiple"]


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _run(g, dev, requires_grad=False, ckpt=0):
    from seistorch_gb300 import engine
    nz, nx = g["models"]["vp"].shape
    prop = engine.BornPropagator(nz, nx, g["dt"], g["h"], g["order"], g["width"], g["multiple"], dev)
    vp = torch.tensor(g["models"]["vp"], dtype=torch.float32, device=dev)
    m = torch.tensor(g["models"]["m"], dtype=torch.float32, device=dev, requires_grad=requires_grad)
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    rec = engine.born_loop(vp, m, prop, d, acq, ckpt)
    B = len(g["sources"])
    nrec = len(g["receivers"][0][0])
    per_shot = rec.reshape(g["nt"], B, nrec, 1).permute(1, 0, 2, 3)
    return m, per_shot


@pytest.mark.parametrize("name", BORN_CASES)
def test_born_records_match_reference(dev, name):
    g = load(name)
    _, rec = _run(g, dev)
    got = rec.detach().cpu().numpy()
    assert got.shape == g["records"].shape
    assert rel_l2(got, g["records"]) < 1e-5
    assert rel_l2(got, g["records_f32"]) < 1e-5


@pytest.mark.parametrize("name", BORN_GRAD_CASES)
@pytest.mark.parametrize("ckpt", [0, 25])
def test_born_gradient_matches_reference_autograd(dev, name, ckpt):
    """dJ/dm through the HABC adjoint of the scattered field against the
    reconstructed background, vs the reference's autograd gradient."""
    g = load(name)
    m, rec = _run(g, dev, requires_grad=True, ckpt=ckpt)
    obs = torch.tensor(g["obs"], dtype=torch.float32, device=dev)
    loss = ((rec - obs) ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    w = g["width"]
    box = (slice(0 if g["multiple"] else w, -w), slice(w, -w))
    got = m.grad.cpu().numpy()
    assert rel_l2(got[box], g["grad_m"][box]) < 1e-4
    mask = np.ones_like(got, bool)
    mask[box] = False
    assert np.all(got[mask] == 0)


def test_born_single_step_matches_oracle(dev):
    """The equation-module drop-in (acoustic_lsrtm_habc._time_step) against
    the oracle's Born step on random fields."""
    from seistorch_gb300.equations2d import acoustic_lsrtm_habc as mod
    g = load("born_habc_o2")
    mod.spatial_order = g["order"]
    rng = np.random.default_rng(1)
    nz, nx = g["models"]["vp"].shape
    f = [rng.standard_normal((2, nz, nx)).astype(np.float32) for _ in range(4)]
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    p0, h1, s0, sh1 = mod._time_step(t(g["models"]["vp"]), t(g["models"]["m"]), *[t(a) for a in f],
                                     torch.tensor(g["dt"]), torch.tensor(g["h"]), t(g["d"]), habcs=(1, 1, 1, 1))
    want = fd2d.born_habc_step(g["models"]["vp"], g["models"]["m"], *f, g["dt"], g["h"], g["d"], 2)
    assert rel_l2(p0.cpu().numpy(), want[0]) < 2e-6
    assert rel_l2(s0.cpu().numpy(), want[2]) < 2e-6
    assert torch.equal(h1.cpu(), torch.tensor(f[0])) and torch.equal(sh1.cpu(), torch.tensor(f[2]))


def test_born_through_wavernn(dev):
    """The user path: build_model(dict config, acoustic_lsrtm_habc) ->
    WaveRNN records of sh1, differentiable in m."""
    from seistorch_gb300 import build_model
    g = load("born_habc_o2")
    w = g["width"]
    vp_int = g["models"]["vp"][w:-w, w:-w]
    m_int = g["models"]["m"][w:-w, w:-w]
    cfg = {"equation": "acoustic_lsrtm_habc", "dtype": "float32",
           "geom": {"dt": g["dt"], "h": g["h"], "nt": g["nt"], "boundary": {"type": "habc", "width": w},
                    "multiple": False, "boundary_saving": True, "source_type": ["h1"],
                    "receiver_type": ["sh1"], "spatial_order": 2, "invlist": {"vp": False, "m": True}}}
    _, model = build_model(cfg, device=dev, mode="inversion", models={"vp": vp_int, "m": m_int})
    srcs = [[int(x) - w, int(z) - w] for z, x in g["src"]]
    recs = [[[int(x) - w for x in xs], [int(z) - w for z in zs]] for zs, xs in g["receivers"]]
    model.reset_geom([0, 1], srcs, recs, cfg)
    y = model(torch.tensor(g["wavelet"])[None])
    got = np.stack([t.detach().cpu().numpy() for t in y])
    assert rel_l2(got, g["records"]) < 1e-5
    sum(t.pow(2).sum() for t in y).backward()
    assert model.cell.geom.m.grad is not None and torch.isfinite(model.cell.geom.m.grad).all()
