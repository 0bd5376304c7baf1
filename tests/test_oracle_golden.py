"""Pin the CPU oracle against vectors produced by the reference's own code."""
import numpy as np
import pytest

from oracle import fd2d
from tests.golden_cases import FORWARD_CASES, load, rel_l2


@pytest.mark.parametrize("name", FORWARD_CASES)
def test_oracle_forward_matches_reference_fp64(name):
    g = load(name)
    eq = g["equation"]
    nz, nx = g["models"]["vp"].shape
    # coefficient generators (pml.py:29-59 / habc.py:42-81) match bit-for-bit in fp64
    if g["habc"]:
        d = fd2d.habc_coefficients_2d((nz, nx), g["width"], g["multiple"])
    else:
        d = fd2d.pml_profile_2d((nz, nx), g["width"], g["multiple"])
    np.testing.assert_allclose(d, g["d"], rtol=1e-14, atol=1e-12)
    out = fd2d.forward(eq, g["models"], g["d"], g["dt"], g["h"], g["wavelet"], g["sources"],
                       g["receivers"], order=g["order"], multiple=g["multiple"],
                       source_type=g["source_type"], receiver_type=g["receiver_type"],
                       return_fields=True)
    rec = np.stack(out["records"])
    assert rec.shape == g["records"].shape
    assert rel_l2(rec, g["records"]) < 1e-11
    for n in fd2d.WAVEFIELDS[eq]:
        assert rel_l2(out["fields"][n][0], g["field_" + n]) < 1e-10, n


def test_oracle_born_records_are_the_scattered_field():
    """The Born records (receivers on sh1) vanish with m = 0 and are linear
    in m: the oracle at 2m gives twice the records."""
    g = load("born_habc_o2")
    args = (g["d"], g["dt"], g["h"], g["wavelet"], g["sources"], g["receivers"])
    kw = dict(order=2, source_type=["h1"], receiver_type=["sh1"], nt=80)
    zero = {"vp": g["models"]["vp"], "m": np.zeros_like(g["models"]["m"])}
    r0 = np.stack(fd2d.forward("acoustic_lsrtm_habc", zero, *args, **kw)["records"])
    assert np.abs(r0).max() == 0.0
    r1 = np.stack(fd2d.forward("acoustic_lsrtm_habc", g["models"], *args, **kw)["records"])
    twice = {"vp": g["models"]["vp"], "m": 2.0 * g["models"]["m"]}
    r2 = np.stack(fd2d.forward("acoustic_lsrtm_habc", twice, *args, **kw)["records"])
    assert np.abs(r1).max() > 0.0
    assert rel_l2(r2, 2.0 * r1) < 1e-12


@pytest.mark.parametrize("name", ["acoustic_pml_o4", "acoustic_habc_o2", "elastic"])
def test_oracle_fp32_tracks_reference_fp32(name):
    """The oracle in float32 stays as close to the reference fp32 run as
    the two fp32 runs are to fp64 (a sanity check of the fp32 mode used by
    the CPU baseline)."""
    g = load(name)
    out = fd2d.forward(g["equation"], g["models"], g["d"], g["dt"], g["h"], g["wavelet"],
                       g["sources"], g["receivers"], order=g["order"], multiple=g["multiple"],
                       dtype=np.float32)
    rec = np.stack(out["records"])
    assert rel_l2(rec, g["records"]) < 1e-4
    assert rel_l2(g["records_f32"], g["records"]) < 1e-4


def test_ricker_and_padding():
    w = fd2d.ricker(10.0, 0.001, 200, delay=100)
    assert w.dtype == np.float32 and abs(w[100] - 1.0) < 1e-7
    m = np.arange(12.0).reshape(3, 4)
    p = fd2d.pad_model(m, 2)
    assert p.shape == (7, 8) and p[0, 0] == m[0, 0] and p[-1, -1] == m[-1, -1]
    p = fd2d.pad_model(m, 2, multiple=True)
    assert p.shape == (5, 8)


def test_fd_coefficients_known_values():
    np.testing.assert_allclose(fd2d.fd_coefficients(2), [1.0])
    np.testing.assert_allclose(fd2d.fd_coefficients(4), [4 / 3, -1 / 12])
    np.testing.assert_allclose(fd2d.fd_coefficients(8), [8 / 5, -1 / 5, 8 / 315, -1 / 560])
