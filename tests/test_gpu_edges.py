"""Edge cases of the GPU path against the fp64 oracle: grids whose width is
not a multiple of 4 (pitched rows with padding columns), duplicate source
points in a shot (injected once, as the reference's 0/1 mask), a shot
without receivers, receivers on the grid's edges, a single time step, one
wavelet row per source (source encoding).  Tolerances as elsewhere:
records 1e-5, gradients inside the undamped box 1e-4 (relative L2)."""
import numpy as np
import pytest
import torch

from oracle import adjoint, fd2d
from tests.golden_cases import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _model(nz, nx, w, seed, lo=1600.0, hi=2600.0):
    rng = np.random.default_rng(seed)
    v = lo + (hi - lo) * rng.random((nz, nx))
    v = (v + np.roll(v, 1, 0) + np.roll(v, 1, 1) + np.roll(v, -1, 1)) / 4
    return fd2d.pad_model(v, w)


def _split(rec, counts, nch=1):
    """records (nt, sum nrec, nch) -> per-shot list."""
    out, k = [], 0
    for c in counts:
        out.append(rec[:, k:k + c])
        k += c
    return out


def test_acoustic_odd_width_edges_and_duplicates(dev):
    from seistorch_gb300 import engine
    w = 12
    vp = _model(25, 35, w, 0)  # padded 49 x 59: pitch 60
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    nt, dt, h = 160, 0.001, 10.0
    wav = fd2d.ricker(18.0, dt, nt, delay=50)
    src = [[(w + 2, w + 3), (w + 2, w + 3), (w + 5, nx - w - 2)], [(nz - w - 3, w + 20)], [(w + 1, w + 10)]]
    rec = [([0, nz - 1, w + 1, w + 1], [0, nx - 1, w, nx - w - 1]), ([], []),
           ([w + 1] * 7, list(range(w, w + 35, 5)))]
    want = fd2d.forward("acoustic", {"vp": vp}, d, dt, h, wav, src, rec, order=4)["records"]
    prop = engine.AcousticPropagator(nz, nx, dt, h, 4, "pml", w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    vpt = torch.tensor(vp, dtype=torch.float32, device=dev, requires_grad=True)
    r, _ = engine.acoustic_loop(vpt, prop, torch.tensor(d, dtype=torch.float32, device=dev), acq, False, 40)
    got = _split(r.detach().cpu().numpy(), acq.reccounts)
    for g_, w_ in zip(got, want):
        if w_.size:
            assert rel_l2(g_, w_) < 1e-5
        else:
            assert g_.size == 0
    (r ** 2).sum().backward()
    resid = [2.0 * x.astype(np.float64) for x in got]
    g_ref = adjoint.acoustic_pml_gradient(vp, d, dt, h, wav, src, rec, resid, order=4)
    box = (slice(w, nz - w), slice(w, nx - w))
    assert rel_l2(vpt.grad.cpu().numpy()[box], g_ref[box]) < 1e-4


def test_habc_odd_width(dev):
    from seistorch_gb300 import engine
    vp = _model(10, 23, 50, 1)  # padded 110 x 123: pitch 124
    nz, nx = vp.shape
    b = fd2d.habc_coefficients_2d((nz, nx), 50)
    nt, dt, h = 180, 0.001, 10.0
    wav = fd2d.ricker(15.0, dt, nt, delay=60)
    src = [[(52, 55)], [(54, 70)]]
    rec = [([51] * 23, list(range(50, 73)))] * 2
    want = fd2d.forward("acoustic_habc", {"vp": vp}, b, dt, h, wav, src, rec, order=4)["records"]
    prop = engine.AcousticPropagator(nz, nx, dt, h, 4, "habc", 50, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    r, _ = engine.acoustic_loop(torch.tensor(vp, dtype=torch.float32, device=dev), prop,
                                torch.tensor(b, dtype=torch.float32, device=dev), acq)
    got = _split(r.cpu().numpy(), acq.reccounts)
    for g_, w_ in zip(got, want):
        assert rel_l2(g_, w_) < 1e-5


def test_elastic_odd_width_and_source_on_velocity(dev):
    from seistorch_gb300 import elastic_engine, engine
    w = 10
    vp = _model(22, 33, w, 2, 2200.0, 3200.0)  # padded 42 x 53: pitch 56
    vs, rho = vp / 1.73, 310.0 * vp ** 0.25
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    nt, dt, h = 150, 0.0005, 5.0
    wav = fd2d.ricker(25.0, dt, nt, delay=40)
    src = [[(w + 2, w + 4)], [(w + 6, nx - w - 3)]]
    rec = [([w + 1] * 11, list(range(w, w + 33, 3))), ([nz - 1, 0], [nx - 1, 0])]
    st, rt = ["vz"], ["vx", "vz", "txx"]
    mod = {"vp": vp, "vs": vs, "rho": rho}
    want = fd2d.forward("elastic", mod, d, dt, h, wav, src, rec, source_type=st, receiver_type=rt)["records"]
    prop = elastic_engine.ElasticPropagator(nz, nx, dt, h, w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    io, nch = elastic_engine.make_io(st, rt)
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev, requires_grad=True)
    m = [t(vp), t(vs), t(rho)]
    r, _ = elastic_engine.elastic_records(*m, prop, torch.tensor(d, dtype=torch.float32, device=dev), acq, io,
                                          nch, False, 40)
    got = _split(r.detach().cpu().numpy(), acq.reccounts)
    for g_, w_ in zip(got, want):
        assert rel_l2(g_, w_) < 1e-5
    (r ** 2).sum().backward()
    resid = [2.0 * x.astype(np.float64) for x in got]
    ref = adjoint.elastic_gradient(vp, vs, rho, d, dt, h, wav, src, rec, resid, source_type=tuple(st),
                                   receiver_type=tuple(rt))
    box = (slice(w, nz - w), slice(w, nx - w))
    for p, g_ in zip(m, ref):
        assert rel_l2(p.grad.cpu().numpy()[box], g_[box]) < 1e-4


def test_single_step_and_per_source_wavelets(dev):
    """nt = 1, and sources injecting their own wavelet rows (source encoding:
    several sources in one shot, one row each)."""
    from seistorch_gb300 import engine
    w = 8
    vp = _model(16, 30, w, 3)
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    dt, h = 0.001, 10.0
    prop = engine.AcousticPropagator(nz, nx, dt, h, 2, "pml", w, False, dev)
    rec = [([w + 2] * 30, list(range(w, w + 30)))]
    # one step
    wav1 = np.array([[1.0]], np.float32)
    acq = engine.Acquisition(nz, nx, [[(w + 2, w + 5)]], rec, wav1, dev)
    r, _ = engine.acoustic_loop(torch.tensor(vp, dtype=torch.float32, device=dev), prop,
                                torch.tensor(d, dtype=torch.float32, device=dev), acq)
    want = fd2d.forward("acoustic", {"vp": vp}, d, dt, h, wav1[0], [[(w + 2, w + 5)]], rec)["records"][0]
    assert rel_l2(r.cpu().numpy(), want) < 1e-6
    # two sources with different wavelets in one shot (superposition of two runs)
    nt = 120
    wa = fd2d.ricker(15.0, dt, nt, delay=40)
    wb = -0.5 * fd2d.ricker(10.0, dt, nt, delay=70)
    srcs = [(w + 2, w + 5), (w + 9, w + 22)]
    acq2 = engine.Acquisition(nz, nx, [srcs], rec, np.stack([wa, wb]), dev, src_wrow=[[0, 1]])
    r2, _ = engine.acoustic_loop(torch.tensor(vp, dtype=torch.float32, device=dev), prop,
                                 torch.tensor(d, dtype=torch.float32, device=dev), acq2)
    ra = fd2d.forward("acoustic", {"vp": vp}, d, dt, h, wa, [[srcs[0]]], rec)["records"][0]
    rb = fd2d.forward("acoustic", {"vp": vp}, d, dt, h, wb, [[srcs[1]]], rec)["records"][0]
    assert rel_l2(r2.cpu().numpy(), ra + rb) < 1e-5
