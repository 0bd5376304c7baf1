"""Learned preconditioner on the GPU: the network's forward and backward
(tcgen05 convolutions + SIMT layers) against the CPU oracle, training
reduces the loss, and a short inversion where the network's steps are
judged by the data misfit.

Tolerances (relative L2).  Both sides store bf16 activations and
gradients at the same points, so they differ only where an fp32 sum rounds
to a different bf16 value or a ReLU input lands on the other side of zero.
bf16 storage itself moves this random network's parameter gradients 5-18 %
away from the exact float64 network, so the check is relative to that
noise level: per layer, GPU vs oracle < 0.1 and < 0.75 x (bf16 oracle vs
exact oracle); prediction <= 1e-2."""
import numpy as np
import pytest
import torch

from oracle import unet
from tests.golden_cases import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def test_network_forward_backward_match_oracle(dev):
    from seistorch_gb300.learned import LAYERS, PrecondNet
    net = PrecondNet(dev, seed=3)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((1, 2, 16, 512)).astype(np.float32)
    dpred = rng.standard_normal((1, 16, 512)).astype(np.float32)
    pred = net.forward(torch.tensor(x, device=dev)).cpu().numpy()
    net.zero_grad()
    net.backward(torch.tensor(dpred, device=dev))
    grads = net.grads.cpu().numpy().astype(np.float64)
    params = net.params.cpu().numpy().astype(np.float64)
    want, cache = unet.forward(params, x.astype(np.float64))
    assert rel_l2(pred, want) < 1e-2
    gw = unet.backward(params, cache, dpred.astype(np.float64))
    _, exact = unet.forward(params, x.astype(np.float64), rounding=False)
    g0 = unet.backward(params, exact, dpred.astype(np.float64))
    off = 0
    for name, ci, co, _ in LAYERS:
        sl = slice(off, off + ci * co * 9 + co)
        err = rel_l2(grads[sl], gw[sl])
        noise = rel_l2(gw[sl], g0[sl])
        assert err < 0.1 and err < 0.75 * noise, (name, err, noise)
        off = sl.stop


def test_training_reduces_the_loss(dev):
    from seistorch_gb300.learned import PrecondNet
    net = PrecondNet(dev, seed=0)
    torch.manual_seed(0)
    x = torch.randn(4, 2, 32, 512, device=dev)
    y = 0.5 * x[:, 0] - 0.25 * x[:, 1]  # a local linear map of the inputs
    losses = [float(net.train_batch(x, y, 2e-3)) for _ in range(60)]
    assert losses[-1] < 0.2 * losses[0]
    from seistorch_gb300 import _native
    assert _native.device_status() == 0


def test_inversion_step_is_judged_by_the_misfit(dev):
    """A short inversion on a small survey: the misfit never increases, and
    a network whose output is useless falls back to the plain step."""
    from seistorch_gb300 import fwi
    from seistorch_gb300.learned import PrecondNet
    sv = fwi.Survey(nz=64, nx=512, shots=4, nt=400, fm=12.0, device=dev)
    rng = np.random.default_rng(1)
    vt = fwi.random_model(rng, 64, 512)
    v0 = fwi.smooth(vt)
    obs = sv.records(sv.pad(vt))
    net = PrecondNet(dev, seed=5)
    with torch.no_grad():
        net.params.zero_()  # predicts zero updates: every learned step must be rejected
    net.pack()
    out = fwi.invert(sv, obs, v0, iters=3, net=net)
    assert out["learned_steps"] == 0
    m = out["misfit"]
    assert all(b <= a for a, b in zip(m, m[1:])) and m[-1] < m[0]


def test_trained_network_gains_over_the_plain_method(dev):
    """Train on 64 solver-generated pairs (64 x 512 models, 4 shots, 500
    steps), then invert a held-out model for 3 iterations with and without
    the network: the learned run takes at least one network step and ends
    at a lower data misfit than the plain illumination-preconditioned run."""
    from seistorch_gb300 import fwi
    from seistorch_gb300.learned import PrecondNet
    sv_tr = fwi.Survey(64, 512, shots=4, nt=500, fm=10.0, device=dev)
    X, Y = fwi.make_pairs(64, sv_tr, seed=100)
    net = PrecondNet(dev, seed=0)
    hist = fwi.train(net, X, Y, epochs=25, batch=8, lr=1e-3)
    assert hist[-1] < 0.8 * hist[0]
    sv = fwi.Survey(64, 512, shots=8, nt=600, fm=10.0, device=dev)
    rng = np.random.default_rng(7)
    vt = fwi.random_model(rng, 64, 512)
    v0 = fwi.smooth(vt)
    obs = sv.records(sv.pad(vt))
    plain = fwi.invert(sv, obs, v0, iters=3)
    learned = fwi.invert(sv, obs, v0, iters=3, net=net)
    print("plain", plain["misfit"], "learned", learned["misfit"], learned["learned_steps"])
    assert learned["learned_steps"] >= 1
    assert learned["misfit"][-1] < plain["misfit"][-1]
