"""GPU parity at the headline run length, illumination parity, and the
bounded-wait status path.

* The boundary-saving gradient over 3000 reversed steps (8th order,
  dt = 1 ms, h = 10 m, 8 Hz, velocities 1500-4500 m/s drawn like the
  400x1000 benchmark model: seeded noise, Gaussian filter sigma = 20 cells,
  rescaled) on a reduced 100x200 interior + 50-cell PML with 2 shots, so
  that the float64 oracle adjoint fits in memory.  The fp32 wavefield is
  rebuilt backwards from the saved boundary ring with checkpoints every K
  steps; the gradient inside the undamped box must stay within 1e-4
  (relative L2) of the oracle's with the same residual.  The drift without
  checkpoints (K = nt) is printed beside it.
* Source illumination (sum over steps and shots of the source field squared,
  rnn.py:127-128,204-205) of the acoustic and elastic loops vs the oracle's
  float64 loop, relative L2 <= 1e-5.
* A wait that nothing completes runs out of polls, sets the timeout bit of
  the device status word and returns; the context stays usable.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint, fd2d
from tests.golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _smooth_random_models(nzi, nxi, w, seed):
    """True and starting models with the benchmark model's statistics."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    noise = gaussian_filter(rng.standard_normal((nzi, nxi)), sigma=20)
    noise = (noise - noise.min()) / (noise.max() - noise.min())
    vp_true = 1500.0 + 3000.0 * noise
    vp_init = gaussian_filter(vp_true, sigma=40)
    pad = lambda m: np.pad(m, w, mode="edge")
    return pad(vp_true), pad(vp_init)


def test_gradient_at_headline_length_vs_fp64_oracle(dev):
    from seistorch_gb300 import engine
    nzi, nxi, w, nt, dt, h, order = 100, 200, 50, 3000, 0.001, 10.0, 8
    vp_true, vp_init = _smooth_random_models(nzi, nxi, w, seed=7)
    nz, nx = vp_true.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    wav = fd2d.ricker(8.0, dt, nt, delay=int(1.5 / 8.0 / dt))
    src = [[(w + 2, w + 40)], [(w + 2, w + 160)]]
    rec = [([w + 2] * nxi, list(range(w, w + nxi)))] * 2
    prop = engine.AcousticPropagator(nz, nx, dt, h, order, "pml", w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    dt_ = torch.tensor(d, dtype=torch.float32, device=dev)
    with torch.no_grad():
        obs, _ = engine.acoustic_loop(torch.tensor(vp_true, dtype=torch.float32, device=dev), prop, dt_, acq)
    K = engine.default_ckpt_every(nt)
    grads, resid = {}, None
    for ck in (K, 0):
        vp = torch.tensor(vp_init, dtype=torch.float32, device=dev, requires_grad=True)
        syn, _ = engine.acoustic_loop(vp, prop, dt_, acq, False, ck)
        ((syn - obs) ** 2).sum().backward()
        grads[ck] = vp.grad.cpu().numpy().astype(np.float64)
        r = 2.0 * (syn - obs).detach().cpu().double().numpy().reshape(nt, 2, nxi, 1)
        resid = r if resid is None else resid
        assert np.array_equal(r, resid)  # the forward does not depend on the checkpoint spacing
    want = adjoint.acoustic_pml_gradient(vp_init, d, dt, h, wav, src, rec, [resid[:, b] for b in range(2)],
                                         order=order, keep_every=60)
    box = (slice(w, -w), slice(w, -w))
    err = {ck: rel_l2(g[box], want[box]) for ck, g in grads.items()}
    print(f"nt={nt} o{order}: gradient rel L2 vs fp64 oracle, checkpoints every {K}: {err[K]:.3e}; "
          f"without checkpoints: {err[0]:.3e}")
    assert err[K] < 1e-4


@pytest.mark.parametrize("name", ["acoustic_pml_o4", "acoustic_habc_o2", "acoustic_pml_o4_multiple"])
def test_acoustic_illumination_vs_oracle(dev, name):
    from seistorch_gb300 import engine
    g = load(name)
    vp = g["models"]["vp"]
    nz, nx = vp.shape
    prop = engine.AcousticPropagator(nz, nx, g["dt"], g["h"], g["order"], "habc" if g["habc"] else "pml",
                                     g["width"], g["multiple"], dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    _, illum = engine.acoustic_loop(torch.tensor(vp, dtype=torch.float32, device=dev), prop,
                                    torch.tensor(g["d"], dtype=torch.float32, device=dev), acq, True)
    want = fd2d.forward("acoustic_habc" if g["habc"] else "acoustic", {"vp": vp}, g["d"], g["dt"], g["h"],
                        g["wavelet"], g["sources"], g["receivers"], order=g["order"], multiple=g["multiple"],
                        illumination=True)["illum"]
    assert illum.shape == want.shape
    assert rel_l2(illum.cpu().numpy(), want) < 1e-5


def test_acoustic_illumination_config1_shape(dev):
    """128x256 + 50-cell PML, 4th order, 1000 steps, 2 shots."""
    from seistorch_gb300 import engine
    nzi, nxi, w, nt = 128, 256, 50, 1000
    vpi = np.zeros((nzi, nxi))
    vpi[:43], vpi[43:86], vpi[86:] = 1500.0, 2500.0, 3500.0
    vp = fd2d.pad_model(vpi, w)
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    wav = fd2d.ricker(10.0, 0.001, nt, delay=100)
    src = [[(w + 2, w + 16)], [(w + 2, w + 144)]]
    rec = [([w + 2] * nxi, list(range(w, w + nxi)))] * 2
    prop = engine.AcousticPropagator(nz, nx, 0.001, 10.0, 4, "pml", w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    _, illum = engine.acoustic_loop(torch.tensor(vp, dtype=torch.float32, device=dev), prop,
                                    torch.tensor(d, dtype=torch.float32, device=dev), acq, True)
    want = fd2d.forward("acoustic", {"vp": vp}, d, 0.001, 10.0, wav, src, rec, order=4, illumination=True)["illum"]
    err = rel_l2(illum.cpu().numpy(), want)
    print(f"illumination 128x256 o4 1000 steps rel L2 vs fp64 oracle: {err:.3e}")
    assert err < 1e-5


@pytest.mark.parametrize("name", ["elastic", "elastic_multiple"])
def test_elastic_illumination_vs_oracle(dev, name):
    from seistorch_gb300 import elastic_engine, engine
    g = load(name)
    m = g["models"]
    nz, nx = m["vp"].shape
    prop = elastic_engine.ElasticPropagator(nz, nx, g["dt"], g["h"], g["width"], g["multiple"], dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    io, nch = elastic_engine.make_io(g["source_type"], g["receiver_type"])
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    _, illum = elastic_engine.elastic_records(t(m["vp"]), t(m["vs"]), t(m["rho"]), prop, t(g["d"]), acq, io, nch,
                                              True)
    want = fd2d.forward("elastic", m, g["d"], g["dt"], g["h"], g["wavelet"], g["sources"], g["receivers"],
                        multiple=g["multiple"], source_type=g["source_type"], receiver_type=g["receiver_type"],
                        illumination=True)["illum"]
    assert rel_l2(illum.cpu().numpy(), want) < 1e-5


def test_bounded_wait_runs_out_and_reports(dev):
    from seistorch_gb300 import _native as N
    from seistorch_gb300 import engine
    lib = N.load()
    N.device_status(reset=True)
    # a barrier that its own thread completes: the wait succeeds, no status bit
    N.check(lib.sgb_debug_wait_probe(64, 1, N.stream_handle()), "sgb_debug_wait_probe")
    torch.cuda.synchronize()
    assert N.device_status(reset=True) == 0
    # nothing completes it: the wait gives up after 64 polls and says so
    N.check(lib.sgb_debug_wait_probe(64, 0, N.stream_handle()), "sgb_debug_wait_probe")
    torch.cuda.synchronize()
    assert N.device_status(reset=True) & 2
    assert lib.sgb_debug_wait_probe(0, 0, N.stream_handle()) == 1
    # the context is still usable: a forward run matches the reference
    g = load("acoustic_pml_o2")
    nz, nx = g["models"]["vp"].shape
    prop = engine.AcousticPropagator(nz, nx, g["dt"], g["h"], g["order"], "pml", g["width"], False, dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    rec, _ = engine.acoustic_loop(torch.tensor(g["models"]["vp"], dtype=torch.float32, device=dev), prop,
                                  torch.tensor(g["d"], dtype=torch.float32, device=dev), acq)
    B, nrec = len(g["sources"]), len(g["receivers"][0][0])
    got = rec.reshape(g["nt"], B, nrec, 1).permute(1, 0, 2, 3).cpu().numpy()
    assert rel_l2(got, g["records"]) < 1e-5
    assert N.device_status(reset=True) == 0
