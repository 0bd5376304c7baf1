"""GPU parity of the variable-density acoustic equation with the HABC
(acoustic_rho_habc: one-cell differences weighted by averaged buoyancies,
C = dt^2 rho vp^2 / h^2, then the one-way-wave blend) against the
reference's own outputs (golden vectors made by tests/golden/make_golden.py)
and the fp64 oracle.

Tolerances (relative L2): records vs the reference in fp64 <= 1e-5; vp and
rho gradients inside the undamped box vs the reference's autograd gradient
<= 1e-4, and 0 outside it.
"""
import numpy as np
import pytest
import torch

from oracle import fd2d
from tests.golden_cases import RHO_GRAD_CASES, load, rel_l2

pytestmark = pytest.mark.gpu

NAMES = ("vp", "rho")


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
    prop = engine.RhoPropagator(nz, nx, g["dt"], g["h"], g["width"], g["multiple"], dev)
    ms = [torch.tensor(g["models"][n], dtype=torch.float32, device=dev, requires_grad=requires_grad) for n in NAMES]
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    rec = engine.rho_loop(*ms, prop, d, acq, ckpt)
    B = len(g["sources"])
    nrec = len(g["receivers"][0][0])
    return ms, rec.reshape(g["nt"], B, nrec, 1).permute(1, 0, 2, 3)


@pytest.mark.parametrize("name", ["rho_habc", "rho_habc_multiple"])
def test_rho_records_match_reference(dev, name):
    g = load(name)
    _, rec = _run(g, dev)
    got = rec.detach().cpu().numpy()
    assert got.shape == g["records"].shape
    assert rel_l2(got, g["records"]) < 1e-5
    assert rel_l2(got, g["records_f32"]) < 1e-5


@pytest.mark.parametrize("name", RHO_GRAD_CASES)
@pytest.mark.parametrize("ckpt", [0, 25])
def test_rho_gradients_match_reference_autograd(dev, name, ckpt):
    """The five coefficient gradients of the variable-density HABC adjoint,
    chained through the coefficient map to vp and rho."""
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


def test_rho_single_step_matches_oracle(dev):
    from seistorch_gb300.equations2d import acoustic_rho_habc as mod
    g = load("rho_habc")
    rng = np.random.default_rng(3)
    nz, nx = g["models"]["vp"].shape
    p1, p2 = [rng.standard_normal((2, nz, nx)).astype(np.float32) for _ in range(2)]
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    y, p1o = mod._time_step(*[t(g["models"][n]) for n in NAMES], t(p1), t(p2), torch.tensor(g["dt"]),
                            torch.tensor(g["h"]), t(g["d"]), habcs=(1, 1, 1, 1))
    want, _ = fd2d.rho_habc_step(g["models"]["vp"], g["models"]["rho"], p1, p2, g["dt"], g["h"], g["d"])
    assert rel_l2(y.cpu().numpy(), want) < 2e-6
    assert torch.equal(p1o.cpu(), torch.tensor(p1))
