"""GPU parity of the VTI acoustic equation with the HABC (vti_habc2: x and z
coefficient planes from vp, eps, delta and the reference's per-cell sk,
then the one-way-wave blend) against the reference's own outputs (golden
vectors made by tests/golden/make_golden.py) and the fp64 oracle.

Tolerances (relative L2): records vs the reference in fp64 <= 1e-5;
vp / eps / delta gradients inside the undamped box vs the reference's
autograd gradient <= 1e-4, and 0 outside it.
"""
import numpy as np
import pytest
import torch

from oracle import fd2d
from tests.golden_cases import VTI_GRAD_CASES, load, rel_l2

pytestmark = pytest.mark.gpu

NAMES = ("vp", "epsilon", "delta")


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
    prop = engine.VTIPropagator(nz, nx, g["dt"], g["h"], g["width"], g["multiple"], dev)
    ms = [torch.tensor(g["models"][n], dtype=torch.float32, device=dev, requires_grad=requires_grad) for n in NAMES]
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    rec = engine.vti_loop(*ms, prop, d, acq, ckpt)
    B = len(g["sources"])
    nrec = len(g["receivers"][0][0])
    return ms, rec.reshape(g["nt"], B, nrec, 1).permute(1, 0, 2, 3)


@pytest.mark.parametrize("name", ["vti_habc2", "vti_habc2_multiple"])
def test_vti_records_match_reference(dev, name):
    g = load(name)
    _, rec = _run(g, dev)
    got = rec.detach().cpu().numpy()
    assert got.shape == g["records"].shape
    assert rel_l2(got, g["records"]) < 1e-5
    assert rel_l2(got, g["records_f32"]) < 1e-5


@pytest.mark.parametrize("name", VTI_GRAD_CASES)
@pytest.mark.parametrize("ckpt", [0, 25])
def test_vti_gradients_match_reference_autograd(dev, name, ckpt):
    """dJ/dkx, dJ/dkz from the anisotropic HABC adjoint, chained through the
    coefficient map to vp, eps and delta."""
    g = load(name)
    ms, rec = _run(g, dev, requires_grad=True, ckpt=ckpt)
    loss = (rec ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    w = g["width"]
    box = (slice(0 if g["multiple"] else w, -w), slice(w, -w))
    for n, m in zip(NAMES, ms):
        got = m.grad.cpu().numpy()
        assert rel_l2(got[box], g["grad_" + n][box]) < 1e-4, n
        mask = np.ones_like(got, bool)
        mask[box] = False
        assert np.all(got[mask] == 0), n


def test_vti_single_step_matches_oracle(dev):
    from seistorch_gb300.equations2d import vti_habc2 as mod
    g = load("vti_habc2")
    rng = np.random.default_rng(2)
    nz, nx = g["models"]["vp"].shape
    p1, p2 = [rng.standard_normal((2, nz, nx)).astype(np.float32) for _ in range(2)]
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    y, p1o = mod._time_step(*[t(g["models"][n]) for n in NAMES], t(p1), t(p2), torch.tensor(g["dt"]),
                            torch.tensor(g["h"]), t(g["d"]), habcs=(1, 1, 1, 1))
    want, _ = fd2d.vti_habc_step(g["models"]["vp"], g["models"]["epsilon"], g["models"]["delta"], p1, p2,
                                 g["dt"], g["h"], g["d"])
    assert rel_l2(y.cpu().numpy(), want) < 2e-6
    assert torch.equal(p1o.cpu(), torch.tensor(p1))


def test_vti_through_wavernn(dev):
    from seistorch_gb300 import build_model
    g = load("vti_habc2")
    w = g["width"]
    ints = {n: g["models"][n][w:-w, w:-w] for n in NAMES}
    cfg = {"equation": "vti_habc2", "dtype": "float32",
           "geom": {"dt": g["dt"], "h": g["h"], "nt": g["nt"], "boundary": {"type": "habc", "width": w},
                    "multiple": False, "boundary_saving": True, "source_type": ["p1"],
                    "receiver_type": ["p1"], "spatial_order": 2,
                    "invlist": {"vp": True, "epsilon": True, "delta": True}}}
    _, model = build_model(cfg, device=dev, mode="inversion", models=ints)
    srcs = [[int(x) - w, int(z) - w] for z, x in g["src"]]
    recs = [[[int(x) - w for x in xs], [int(z) - w for z in zs]] for zs, xs in g["receivers"]]
    model.reset_geom([0, 1], srcs, recs, cfg)
    y = model(torch.tensor(g["wavelet"])[None])
    got = np.stack([t.detach().cpu().numpy() for t in y])
    assert rel_l2(got, g["records"]) < 1e-5
    sum(t.pow(2).sum() for t in y).backward()
    for n in NAMES:
        gr = getattr(model.cell.geom, n).grad
        assert gr is not None and torch.isfinite(gr).all()
