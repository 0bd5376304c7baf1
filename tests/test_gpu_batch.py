"""Uneven batch: several grids with different shapes, shot counts and trace
lengths in one persistent launch per step, and the same loop replayed from a
CUDA graph.  Each grid's records must equal the single-grid loop's records
exactly (same kernel arithmetic per tile) and match the fp64 oracle."""
import numpy as np
import pytest
import torch

from oracle import fd2d
from tests.golden_cases import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _group(dev, nzi, nxi, nshots, nt, seed, w=20, order=4):
    from seistorch_gb300 import engine
    rng = np.random.default_rng(seed)
    vpi = 1800.0 + 1500.0 * rng.random((nzi, nxi))
    vpi = (vpi + np.roll(vpi, 1, 0) + np.roll(vpi, 1, 1)) / 3
    vp = fd2d.pad_model(vpi, w)
    nz, nx = vp.shape
    d = fd2d.pml_profile_2d((nz, nx), w)
    wav = fd2d.ricker(15.0, 0.001, nt, delay=60)
    xs = np.linspace(w, nx - w - 1, nshots).round().astype(int)
    src = [[(w + 2, int(x))] for x in xs]
    rec = [([w + 2] * nxi, list(range(w, w + nxi)))] * nshots
    prop = engine.AcousticPropagator(nz, nx, 0.001, 10.0, order, "pml", w, False, dev)
    acq = engine.Acquisition(nz, nx, src, rec, wav, dev)
    t = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    return prop, t(vp), t(d), acq, (vp, d, wav, src, rec)


def test_uneven_batch_equals_single_grid_loops(dev):
    from seistorch_gb300 import engine
    specs = [(40, 90, 3, 150, 0), (61, 133, 2, 230, 1), (33, 257, 4, 90, 2)]
    groups = [_group(dev, *s) for s in specs]
    batch = engine.UnevenBatch([g[:4] for g in groups])
    got = batch.run()
    for (prop, vp, d, acq, host), r in zip(groups, got):
        want, _ = engine.acoustic_loop(vp, prop, d, acq)
        assert torch.equal(r, want)
    # graph replays start from zero state and give the same records
    batch.plan()
    for _ in range(2):
        again = batch.replay()
        for a, b in zip(again, got):
            assert torch.equal(a, b)
    batch.close()


def test_uneven_batch_matches_fp64_oracle(dev):
    from seistorch_gb300 import engine
    specs = [(30, 70, 2, 120, 3), (45, 100, 1, 200, 4)]
    groups = [_group(dev, *s) for s in specs]
    got = engine.UnevenBatch([g[:4] for g in groups]).run()
    for (prop, vp, d, acq, (vph, dh, wav, src, rec)), r in zip(groups, got):
        want = np.stack(fd2d.forward("acoustic", {"vp": vph}, dh, 0.001, 10.0, wav, src, rec, order=4)["records"])
        B = len(src)
        g = r.cpu().numpy().reshape(acq.nt, B, -1, 1).transpose(1, 0, 2, 3)
        assert rel_l2(g, want) < 1e-5
