"""GPU parity of the per-step drop-ins (the equation modules' three entry
points) against the reference's own modules run in float64
(tests/golden/make_step_golden.py):

* ``_time_step`` outputs, and their VJP through autograd -- what the
  reference's ``WaveCell`` differentiates every step with
  ``boundary_saving: false`` (cell.py:74-75);
* ``_time_step_backward(_multiple)`` outputs (the unblended reverse update,
  strips restored, source re-added) and their VJP -- what
  ``CheckpointFunction.backward`` differentiates (checkpoint_new.py:180-199);
  the elastic reverse step (elastic.py:39-207) for its outputs.

Tolerances (relative L2, fp32 kernels vs the float64 reference): outputs
1e-6, VJPs 1e-5 (gradients of every model parameter and input field over
the whole grid, strips included).  A per-step loop through the repo's
``WaveCell`` under autograd reproduces the reference's pure-autograd HABC
gradient golden to 1e-4 inside the undamped box.
"""
import glob
import os

import numpy as np
import pytest
import torch

from tests.golden_cases import GOLDEN, load, rel_l2

pytestmark = pytest.mark.gpu

CASES = sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "steps_*.npz")))


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def _case(name):
    z = np.load(os.path.join(GOLDEN, f"steps_{name}.npz"))
    g = {k: z[k] for k in z.files}
    g["equation"] = str(g["equation"])
    g["model_names"] = [str(s) for s in g["model_names"]]
    g["field_names"] = [str(s) for s in g["field_names"]]
    g["src_type"] = [str(s) for s in g["src_type"]]
    for k in ("order",):
        g[k] = int(g[k])
    for k in ("habc", "multiple"):
        g[k] = bool(g[k])
    return g


@pytest.fixture(autouse=True)
def _keep_spatial_orders():
    """The equation modules keep their spatial order in a module global (as
    the reference's do); restore every one after each test so that later
    tests see the default."""
    from seistorch_gb300.equations2d import (acoustic, acoustic_habc, acoustic_lsrtm_habc, acoustic_rho_habc,
                                             vacoustic_habc, vti_habc2)
    mods = [acoustic, acoustic_habc, acoustic_lsrtm_habc, acoustic_rho_habc, vacoustic_habc, vti_habc2]
    saved = [getattr(m, "spatial_order", None) for m in mods]
    yield
    for m, v in zip(mods, saved):
        if v is not None:
            m.spatial_order = v


def _module(g):
    from seistorch_gb300.equations2d import (acoustic, acoustic_habc, acoustic_lsrtm_habc, acoustic_rho_habc,
                                             elastic, vacoustic_habc, vti_habc2)
    mod = {"acoustic": acoustic, "acoustic_habc": acoustic_habc, "acoustic_lsrtm_habc": acoustic_lsrtm_habc,
           "vti_habc2": vti_habc2, "acoustic_rho_habc": acoustic_rho_habc, "vacoustic_habc": vacoustic_habc,
           "elastic": elastic}[g["equation"]]
    if hasattr(mod, "spatial_order"):
        mod.spatial_order = g["order"]
    return mod


def _masks(g, dev):
    if not g["habc"]:
        return None
    from seistorch_gb300.habc import bound_mask
    B, nz, nx = g["in_" + g["field_names"][0]].shape
    return bound_mask(nz, nx, 50, dev, B, return_idx=True, multiple=g["multiple"])


def _inputs(g, dev):
    t = lambda a: torch.tensor(a, dtype=torch.float64, device=dev, requires_grad=True)
    models = [t(g["model_" + n]) for n in g["model_names"]]
    fields = [t(g["in_" + f]) for f in g["field_names"]]
    scal = lambda v: torch.tensor(float(v), dtype=torch.float64, device=dev)
    geo = (scal(g["dt"]), scal(g["h"]), torch.tensor(g["d"], dtype=torch.float64, device=dev))
    return models, fields, geo


def _new_levels(g):
    return sorted(int(k[len("gy_"):]) for k in g if k.startswith("gy_"))


@pytest.mark.parametrize("name", CASES)
def test_time_step_and_its_vjp_match_reference(dev, name):
    g = _case(name)
    mod = _module(g)
    models, fields, geo = _inputs(g, dev)
    out = mod._time_step(*models, *fields, *geo, habcs=_masks(g, dev))
    idx = _new_levels(g)
    for i in idx:
        assert rel_l2(out[i].detach().cpu().numpy(), g[f"step_out_{i}"]) < 1e-6, (name, i)
    loss = sum((out[i] * torch.tensor(g[f"gy_{i}"], dtype=torch.float64, device=dev)).sum() for i in idx)
    loss.backward()
    for n, t in zip(g["model_names"] + g["field_names"], models + fields):
        assert t.grad is not None, n
        err = rel_l2(t.grad.cpu().numpy(), g["step_grad_" + n])
        assert err < 1e-5, (name, n, err)


@pytest.mark.parametrize("name", CASES)
def test_reverse_step_and_its_vjp_match_reference(dev, name):
    g = _case(name)
    mod = _module(g)
    models, fields, geo = _inputs(g, dev)
    strips = [tuple(torch.tensor(g[f"strip_{f}_{k}"], dtype=torch.float64, device=dev) for k in "tblr")
              for f in g["field_names"]]
    smask = torch.tensor(g["smask"], dtype=torch.float64, device=dev)
    sval = torch.tensor(g["src_value"], dtype=torch.float64, device=dev)

    def src_func(Y, X, dt=1.0):
        return Y + smask * X

    back = mod._time_step_backward_multiple if g["multiple"] and g["equation"] != "elastic" \
        else mod._time_step_backward
    out = back(*models, *fields, *geo, strips, [g["src_type"], src_func, sval])
    idx = _new_levels(g)
    for i in idx:
        assert rel_l2(out[i].detach().cpu().numpy(), g[f"rev_out_{i}"]) < 1e-6, (name, i)
    if g["equation"] == "elastic":
        return
    loss = sum((out[i] * torch.tensor(g[f"gy_{i}"], dtype=torch.float64, device=dev)).sum() for i in idx)
    loss.backward()
    for n, t in zip(g["model_names"] + g["field_names"], models + fields):
        want = g["rev_grad_" + n]
        got = t.grad.cpu().numpy() if t.grad is not None else np.zeros_like(want)
        err = rel_l2(got, want) if np.linalg.norm(want) > 0 else float(np.abs(got).max())
        assert err < 1e-5, (name, n, err)


@pytest.mark.parametrize("name", ["grad_acoustic_habc_o2_zeroobs", "grad_acoustic_habc_o2_multiple_zeroobs"])
def test_per_step_loop_through_wavecell_matches_reference_autograd(dev, name):
    """The reference's per-step integration (rnn.py:178-205 calling
    cell.py:74-75 with ``boundary_saving: false``) driven through this
    package's ``WaveCell`` and ``acoustic_habc`` module: autograd through
    every native step and its native VJP gives the reference's autograd
    gradient inside the undamped box (and its loss)."""
    from seistorch_gb300.cell import WaveCell
    from seistorch_gb300.equations2d import acoustic_habc
    g = load(name)
    acoustic_habc.spatial_order = g["order"]
    vp = torch.tensor(g["models"]["vp"], dtype=torch.float32, device=dev, requires_grad=True)
    nz, nx = vp.shape

    class _Geom(torch.nn.Module):
        pass

    geom = _Geom()
    geom.vp = vp
    geom.dt, geom.h = g["dt"], torch.tensor(g["h"], device=dev)
    geom.d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    geom.domain_shape, geom.bwidth, geom.multiple, geom.use_habc = (nz, nx), 50, g["multiple"], True
    geom.boundary_saving, geom.inversion = False, True
    cell = WaveCell(geom, acoustic_habc._time_step, acoustic_habc._time_step_backward).to(dev)
    B = len(g["sources"])
    cell.setup_habc(B)
    smask = torch.zeros(B, nz, nx, device=dev)
    for b, pts in enumerate(g["sources"]):
        for (z, x) in pts:
            smask[b, z, x] = 1.0
    wav = torch.tensor(g["wavelet"], dtype=torch.float32, device=dev)
    h1 = torch.zeros(B, nz, nx, device=dev)
    h2 = torch.zeros(B, nz, nx, device=dev)
    recs = []
    rz = [torch.tensor(r[0], device=dev) for r in g["receivers"]]
    rx = [torch.tensor(r[1], device=dev) for r in g["receivers"]]
    for i in range(g["nt"]):
        h1, h2 = cell([h1, h2], [vp], is_last_frame=i == g["nt"] - 1, source=None)
        h1 = h1 + smask * wav[i]
        recs.append(torch.stack([h1[b, rz[b], rx[b]] for b in range(B)]))
    rec = torch.stack(recs, 1)  # (B, nt, nrec)
    loss = (rec.double() ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    w = g["width"]
    box = (slice(0 if g["multiple"] else w, -w), slice(w, -w))
    assert rel_l2(vp.grad.cpu().numpy()[box], g["grad_vp"][box]) < 1e-4


@pytest.mark.parametrize("name", ["grad_bs_acoustic_pml_o2_zeroobs", "grad_bs_acoustic_habc_o2_zeroobs",
                                  "grad_bs_elastic_zeroobs"])
def test_boundary_saving_wavecell_matches_reference(dev, name):
    """``boundary_saving: true`` inversion through this package's ``WaveCell``
    (the per-step checkpoint protocol of checkpoint_new.py / checkpoint.py
    over the equation modules' native steps and reverse steps), driven the
    way rnn.py:178-205 drives it, reproduces the reference's own
    boundary-saving gradient (relative L2 1e-4 over the whole grid) and loss."""
    from seistorch_gb300.cell import WaveCell
    from seistorch_gb300.eqconfigure import Wavefield
    from seistorch_gb300.equations2d import acoustic, acoustic_habc, elastic
    from seistorch_gb300.source import WaveSource
    from tests.golden_cases import MODEL_PARAMS
    g = load(name)
    eq = g["equation"]
    mod = {"acoustic": acoustic, "acoustic_habc": acoustic_habc, "elastic": elastic}[eq]
    if hasattr(mod, "spatial_order"):
        mod.spatial_order = g["order"]
    names, fields = MODEL_PARAMS[eq], Wavefield(eq).wavefields
    models = [torch.tensor(g["models"][n], dtype=torch.float32, device=dev, requires_grad=True) for n in names]
    nz, nx = models[0].shape
    B = len(g["sources"])

    class _Geom(torch.nn.Module):
        pass

    geom = _Geom()
    geom.dt, geom.h = g["dt"], torch.tensor(g["h"], device=dev)
    geom.d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    geom.domain_shape, geom.bwidth, geom.multiple, geom.use_habc = (nz, nx), g["width"], g["multiple"], g["habc"]
    geom.boundary_saving, geom.inversion = True, True
    cell = WaveCell(geom, mod._time_step, mod._time_step_backward).to(dev)
    if g["habc"]:
        cell.setup_habc(B)
    second = eq != "elastic"
    src = WaveSource(None, second, x=[p[0][1] for p in g["sources"]], y=[p[0][0] for p in g["sources"]]).to(dev)
    src.smask = torch.zeros(B, nz, nx, device=dev)
    for b, pts in enumerate(g["sources"]):
        for (z, x) in pts:
            src.smask[b, z, x] = 1.0
    wav = torch.tensor(g["wavelet"], dtype=torch.float32, device=dev).reshape(1, -1)
    nt = g["nt"]
    state = [torch.zeros(B, nz, nx, device=dev) for _ in fields]
    rz = [torch.tensor(r[0], device=dev) for r in g["receivers"]]
    rx = [torch.tensor(r[1], device=dev) for r in g["receivers"]]
    recs = []
    for i in range(nt):
        tmpi = min(i + (3 if second else 0), nt - 1)
        state = list(cell(state, models, is_last_frame=i == nt - 1,
                          source=[g["source_type"], src, wav[..., tmpi].view(1, -1)]))
        for st in g["source_type"]:
            k = fields.index(st)
            state[k] = src(state[k], wav[..., i].view(1, -1))
        recs.append(torch.stack([torch.stack([state[fields.index(r)][b, rz[b], rx[b]] for r in g["receiver_type"]],
                                             -1) for b in range(B)]))
    rec = torch.stack(recs, 1)
    loss = (rec.double() ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) < 1e-5 * float(g["loss"])
    for n, t in zip(names, models):
        err = rel_l2(t.grad.cpu().numpy(), g["grad_" + n])
        print(f"{name}: d/d{n} rel L2 vs the reference's boundary-saving gradient {err:.3e}")
        assert err < 1e-4, (n, err)
