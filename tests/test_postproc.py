"""Misfit and gradient post-processing: the CPU oracle pinned to golden
vectors made by the reference's own code (tests/golden/make_postproc_golden.py),
and the device kernels against the same vectors (fp32 tolerances:
smoothing / division 1e-6, loss 1e-6 relative)."""
import os

import numpy as np
import pytest
import torch

from oracle import postproc
from tests.golden_cases import GOLDEN, rel_l2


def _g():
    z = np.load(os.path.join(GOLDEN, "postproc.npz"))
    return {k: z[k] for k in z.files}


def _par(g, name):
    sz, rz, sx, rx, c = g["smooth_" + name + "_par"]
    return {"z": float(sz), "x": float(sx)}, {"z": int(rz), "x": int(rx)}, int(c)


def test_oracle_matches_reference_goldens():
    g = _g()
    for name in ("a", "b"):
        sig, rad, c = _par(g, name)
        assert rel_l2(postproc.smooth_gradient(g["grad"], sig, rad, c), g["smooth_" + name]) < 1e-6
    loss, grad = postproc.l2(g["l2_syn"], g["l2_obs"])
    assert abs(loss - float(g["l2_loss"])) < 1e-5 * float(g["l2_loss"])
    assert rel_l2(grad, g["l2_grad"]) < 1e-6


@pytest.mark.gpu
def test_device_post_processing_matches_goldens():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native, postprocess
    _native.load(build_if_missing=False)
    dev = torch.device("cuda:0")
    g = _g()
    t = lambda a: torch.tensor(a, device=dev)
    for name in ("a", "b"):
        sig, rad, c = _par(g, name)
        got = postprocess.smooth_gradient(t(g["grad"]), sig, rad, c).cpu().numpy()
        assert rel_l2(got, g["smooth_" + name]) < 1e-6
    got = postprocess.precondition(t(g["grad"]), t(g["illum"])).cpu().numpy()
    assert rel_l2(got, g["precond"]) < 1e-6
    syn = t(g["l2_syn"]).requires_grad_(True)
    loss = postprocess.L2()(list(syn), list(t(g["l2_obs"])))
    loss.backward()
    assert abs(float(loss) - float(g["l2_loss"])) < 1e-6 * float(g["l2_loss"])
    assert rel_l2(syn.grad.cpu().numpy(), g["l2_grad"]) < 1e-6


@pytest.mark.gpu
def test_steepest_descent_step():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native, postprocess
    _native.load(build_if_missing=False)
    dev = torch.device("cuda:0")
    torch.manual_seed(0)
    p = torch.nn.Parameter(torch.randn(50, 60, device=dev))
    p0 = p.detach().clone()
    p.grad = torch.randn(50, 60, device=dev)
    opt = postprocess.Steepestdescent([p], lr=10.0, grad_clamp=True)
    opt.step()
    q = torch.quantile(p.grad.reshape(-1), torch.tensor([0.02, 0.98], device=dev))
    d = p.grad.clamp(q[0], q[1])
    want = p0 - 10.0 * d / d.abs().max()
    assert torch.allclose(p.detach(), want, rtol=1e-6, atol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("freqs", [5.0, [3.0, 12.0]])
def test_record_filter_matches_scipy_filtfilt(freqs):
    """SeisSignal.filter's scipy backend is scipy.signal.filtfilt(b, a, d,
    axis=0) with a Butterworth design; the device filter matches it to 1e-5
    (both recur in float64; the band-pass design's poles near the unit
    circle amplify the different summation order to ~1e-6)."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from scipy import signal as sps
    from seistorch_gb300 import _native, postprocess
    _native.load(build_if_missing=False)
    rng = np.random.default_rng(0)
    d = rng.standard_normal((500, 37, 2)).astype(np.float32)
    dt = 0.002
    mode = postprocess.filter_mode(freqs)
    f = [freqs] if isinstance(freqs, float) else freqs
    b, a = sps.butter(4, [2 * x * dt for x in f] if len(f) > 1 else 2 * f[0] * dt, btype=mode)
    want = sps.filtfilt(b, a, d, axis=0).astype(np.float32)
    got = postprocess.filter_records(torch.tensor(d, device="cuda"), dt, freqs, 4).cpu().numpy()
    assert rel_l2(got, want) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("tag,beta,clamp", [("pr", "PR", True), ("fr", "FR", False)])
def test_ncg_steps_match_reference(tag, beta, clamp):
    """Four non-linear conjugate-gradient steps (sgb_ncg_step through
    postprocess.Cg) against the reference's Cg optimizer (optimizer.py:144-224)
    on the same parameter and gradients: Polak-Ribiere with the 2 % / 98 %
    quantile clamp, Fletcher-Reeves without it.  The update is lr / max|dir|
    times a float32 direction, so the parameters agree to float32 rounding
    (relative L2 of the change 1e-5)."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    from seistorch_gb300.postprocess import Cg
    _native.load(build_if_missing=False)
    z = np.load(os.path.join(GOLDEN, "postproc.npz"))
    dev = torch.device("cuda:0")
    p = torch.nn.Parameter(torch.tensor(z["ncg_p0"], device=dev))
    opt = Cg([p], lr=10.0, beta_type=beta, grad_clamp=clamp, clip_value=0.02)
    for k in range(4):
        p.grad = torch.tensor(z["ncg_grads"][k], device=dev)
        opt.step()
        want = z["ncg_" + tag][k]
        got = p.detach().cpu().numpy()
        assert rel_l2(got - z["ncg_p0"], want - z["ncg_p0"]) < 1e-5, k
