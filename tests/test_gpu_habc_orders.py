"""GPU parity of the HABC kernels at every compiled variant and order.

* Every variant of the second-order HABC forward (rows per tile, warps,
  stages, previous field via TMA; ``sgb_set_stream_config``'s third
  argument) computes the same arithmetic: identical records, within 1e-5 of
  the reference's (golden ``acoustic_habc_o2``).
* Orders 6 and 8 (no reference golden at these orders): records of the
  HABC loop vs the fp64 oracle (``fd2d.forward``, whose order-8 stencil is
  pinned by the PML goldens and whose HABC blend by the o2 / o4 goldens),
  relative L2 <= 1e-5; and the boundary-saving gradient of J = sum syn^2
  (zero observed data, as the reference's gradient goldens) at single cells
  -- a source, a receiver-row cell, the undamped box's top edge, the
  interior -- vs central differences (J(vp + e d_q) - J(vp - e d_q)) / 2e of
  the oracle's fp64 J, relative error <= 1e-3 (observed: 1e-6 .. 3e-5).
  With nonzero observed data the gradient near a source is the small
  difference of large terms and fp32 residuals cannot resolve it, so the
  zero-data misfit is the well-conditioned probe.
"""
import numpy as np
import pytest
import torch

from oracle import fd2d
from tests.golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu

HABC_FWD_VARIANTS = 6


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native
    _native.load(build_if_missing=False)
    return torch.device("cuda:0")


def test_every_habc_forward_variant_gives_the_same_records(dev):
    from seistorch_gb300 import _native as N
    from seistorch_gb300 import engine, tuning
    g = load("acoustic_habc_o2")
    nz, nx = g["models"]["vp"].shape
    prop = engine.AcousticPropagator(nz, nx, g["dt"], g["h"], g["order"], "habc", g["width"], False, dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)
    vp = torch.tensor(g["models"]["vp"], dtype=torch.float32, device=dev)
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    outs = []
    try:
        for cfg in range(HABC_FWD_VARIANTS):
            N.call("sgb_set_stream_config", tuning.DEFAULT[0], tuning.DEFAULT[1], cfg)
            rec, _ = engine.acoustic_loop(vp, prop, d, acq)
            outs.append(rec.cpu().numpy())
    finally:
        N.call("sgb_set_stream_config", tuning.DEFAULT[0], tuning.DEFAULT[1], 0)
    for o in outs:
        assert np.array_equal(o, outs[0])
    B, nrec = len(g["sources"]), len(g["receivers"][0][0])
    got = outs[0].reshape(g["nt"], B, nrec, 1).transpose(1, 0, 2, 3)
    assert rel_l2(got, g["records"]) < 1e-5


def _case(order):
    """160 x 160 grid (60 x 60 interior + 50-cell HABC), 2 shots, 180 steps."""
    w, nzi, nxi, nt, dt, h = 50, 60, 60, 180, 0.001, 10.0
    nz, nx = nzi + 2 * w, nxi + 2 * w
    zz, xx = np.mgrid[0:nz, 0:nx].astype(np.float64)
    vp0 = 1800.0 + 6.0 * np.clip(zz - w, 0, None) + 150.0 * np.exp(-((zz - 90) ** 2 + (xx - 70) ** 2) / 200.0)
    vp_true = vp0 + 120.0 * np.exp(-((zz - 75) ** 2 + (xx - 85) ** 2) / 60.0)
    b = fd2d.habc_coefficients_2d((nz, nx), w)
    wav = fd2d.ricker(15.0, dt, nt, delay=60)
    src = [[(w + 2, w + 12)], [(w + 2, w + 48)]]
    rec = [([w + 2] * nxi, list(range(w, w + nxi)))] * 2
    return dict(w=w, nt=nt, dt=dt, h=h, order=order, vp0=vp0, vp_true=vp_true, b=b, wav=wav, src=src, rec=rec)


def _oracle_records(c, vp):
    out = fd2d.forward("acoustic_habc", {"vp": vp}, c["b"], c["dt"], c["h"], c["wav"], c["src"], c["rec"],
                       order=c["order"])
    return np.stack(out["records"])  # (B, nt, nrec, 1)


@pytest.mark.parametrize("order", [6, 8])
def test_habc_high_order_records_and_gradient_vs_oracle(dev, order):
    from seistorch_gb300 import engine
    c = _case(order)
    nz, nx = c["vp0"].shape
    B, nrec, nt = 2, len(c["rec"][0][0]), c["nt"]
    prop = engine.AcousticPropagator(nz, nx, c["dt"], c["h"], order, "habc", c["w"], False, dev)
    acq = engine.Acquisition(nz, nx, c["src"], c["rec"], c["wav"], dev)
    bt = torch.tensor(c["b"], dtype=torch.float32, device=dev)
    # records vs the fp64 oracle
    with torch.no_grad():
        r, _ = engine.acoustic_loop(torch.tensor(c["vp_true"], dtype=torch.float32, device=dev), prop, bt, acq)
    got = r.reshape(nt, B, nrec, 1).permute(1, 0, 2, 3).cpu().numpy()
    assert rel_l2(got, _oracle_records(c, c["vp_true"])) < 1e-5
    # the boundary-saving gradient of J = sum syn^2
    vp = torch.tensor(c["vp0"], dtype=torch.float32, device=dev, requires_grad=True)
    syn, _ = engine.acoustic_loop(vp, prop, bt, acq, False, engine.default_ckpt_every(nt))
    (syn.double() ** 2).sum().backward()
    g = vp.grad.double().cpu().numpy()
    J = lambda v: float((_oracle_records(c, v) ** 2).sum())
    e = 1e-2  # m/s
    for (iz, ix) in [(52, 62), (52, 80), (50, 70), (60, 62)]:
        dq = np.zeros_like(c["vp0"])
        dq[iz, ix] = 1.0
        fd = (J(c["vp0"] + e * dq) - J(c["vp0"] - e * dq)) / (2.0 * e)
        print(f"o{order} cell ({iz}, {ix}): gradient {g[iz, ix]:.6e}, central difference {fd:.6e}")
        assert abs(g[iz, ix] - fd) < 1e-3 * abs(fd)
