"""CPU tests: the C-ABI library loads and exports what the header declares,
host-side logic (acquisition tables, config reader, coefficient generators)
matches the reference's semantics.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

from tests.golden_cases import load, rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names.update(re.findall(r"\b(sgb_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from seistorch_gb300 import _native
    _native.build()
    return _native.load()


def test_library_exports_every_declared_symbol(lib):
    syms = _declared_symbols()
    assert len(syms) >= 8
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_host_only_entry_points(lib):
    from seistorch_gb300 import _native as N
    assert b"sm_103a" in lib.sgb_version()
    assert lib.sgb_status_string(0) == b"ok"
    assert lib.sgb_status_string(7).startswith(b"too many")
    g = N.Grid(120, 140, 140, 2, 0.001, 10.0)
    out = ctypes.c_int32(0)
    assert lib.sgb_ring_size(ctypes.byref(g), 50, 70, 50, 90, 4, ctypes.byref(out)) == 0
    # (20+8) x (40+8) box minus the 20 x 40 interior
    assert out.value == 28 * 48 - 20 * 40
    assert lib.sgb_ring_size(ctypes.byref(g), 0, 70, 50, 90, 4, ctypes.byref(out)) == 0
    assert out.value == (70 + 4) * 48 - 70 * 40  # no top band at the free surface
    bad = N.Grid(120, 140, 141, 2, 0.001, 10.0)
    assert lib.sgb_ring_size(ctypes.byref(bad), 50, 70, 50, 90, 4, ctypes.byref(out)) == 3  # pitch % 4
    assert lib.sgb_ring_size(ctypes.byref(g), 50, 70, 50, 90, 0, ctypes.byref(out)) == 1


def test_variant_tables_match_the_abi(lib):
    """Every variant the autotuner names is one sgb_set_stream_config
    accepts, the next index is refused, and the tuner's default is a valid
    pair (host-only: nothing is launched)."""
    from seistorch_gb300 import tuning
    nf, nb = len(tuning.FWD_VARIANTS), len(tuning.BWD_VARIANTS)
    try:
        for f in range(nf):
            assert lib.sgb_set_stream_config(f, 0, 0) == 0, f
        for b in range(nb):
            assert lib.sgb_set_stream_config(0, b, 0) == 0, b
        for h in range(6):
            assert lib.sgb_set_stream_config(0, 0, h) == 0, h
        assert lib.sgb_set_stream_config(nf, 0, 0) != 0
        assert lib.sgb_set_stream_config(0, nb, 0) != 0
        assert lib.sgb_set_stream_config(0, 0, 6) != 0
        assert lib.sgb_set_stream_config(-1, 0, 0) != 0
        assert 0 <= tuning.DEFAULT[0] < nf and 0 <= tuning.DEFAULT[1] < nb
    finally:
        lib.sgb_set_stream_config(tuning.DEFAULT[0], tuning.DEFAULT[1], 0)


def test_calls_validate_before_touching_the_gpu(lib):
    from seistorch_gb300 import _native as N
    g = N.Grid(64, 64, 64, 1, 0.001, 10.0)
    m = N.AcousticModel(3, 0, 50, 0, None, None, None)
    assert lib.sgb_acoustic_step(ctypes.byref(g), ctypes.byref(m), None, None, None, None) == 1
    m = N.AcousticModel(3, 0, 50, 0, ctypes.c_void_p(16), None, None)
    assert lib.sgb_acoustic_step(ctypes.byref(g), ctypes.byref(m), None, None, None, None) == 5
    m = N.AcousticModel(4, 0, 50, 0, ctypes.c_void_p(18), None, None)
    assert lib.sgb_acoustic_step(ctypes.byref(g), ctypes.byref(m), ctypes.c_void_p(16), ctypes.c_void_p(16),
                                 ctypes.c_void_p(32), None) == 3
    g0 = N.Grid(64, 64, 64, 0, 0.001, 10.0)
    assert lib.sgb_acoustic_step(ctypes.byref(g0), ctypes.byref(m), None, None, None, None) == 2


def test_acquisition_tables():
    from seistorch_gb300.engine import Acquisition
    nz, nx = 30, 40
    sources = [[(3, 4), (3, 4), (5, 6)], [(7, 8)]]
    receivers = [([2, 2, 9], [30, 1, 5]), ([4], [4])]
    acq = Acquisition(nz, nx, sources, receivers, np.zeros(10, np.float32), "cpu")
    assert acq.nsrc == 3  # duplicate point injects once (0/1 mask)
    assert acq.src_ptr.tolist() == [0, 2, 3]
    assert acq.nrec == 4 and acq.reccounts == [3, 1]
    ptr = acq.rec_row_ptr.numpy()
    # shot 0 row 2 holds x = 1, 30 (sorted), output columns 1, 0
    s, e = ptr[0 * nz + 2], ptr[0 * nz + 3]
    assert acq.rec_x[s:e].tolist() == [1, 30] and acq.rec_col[s:e].tolist() == [1, 0]
    s, e = ptr[1 * nz + 4], ptr[1 * nz + 5]
    assert acq.rec_col[s:e].tolist() == [3]
    with pytest.raises(IndexError):
        Acquisition(nz, nx, [[(30, 0)]], [([0], [0])], np.zeros(3), "cpu")
    with pytest.raises(IndexError):
        Acquisition(nz, nx, [[(0, 0)]], [([0], [40])], np.zeros(3), "cpu")


@pytest.mark.parametrize("name", ["acoustic_pml_o4", "acoustic_pml_o4_multiple", "acoustic_habc_o2",
                                  "acoustic_habc_o2_multiple"])
def test_boundary_coefficients_match_reference(name):
    from seistorch_gb300 import habc, pml
    g = load(name)
    torch.set_default_dtype(torch.float64)
    try:
        shape = g["models"]["vp"].shape
        if g["habc"]:
            d = habc.generate_habc_coefficients_2d(shape, g["width"], multiple=g["multiple"])
        else:
            d = pml.generate_pml_coefficients_2d(shape, g["width"], multiple=g["multiple"])
    finally:
        torch.set_default_dtype(torch.float32)
    np.testing.assert_allclose(d.numpy(), g["d"], rtol=1e-13, atol=1e-12)


def test_habc_masks_match_oracle():
    from oracle import fd2d
    from seistorch_gb300 import habc
    for multiple in (False, True):
        a = habc.bound_mask(120, 130, 50, "cpu", return_idx=True, multiple=multiple)
        b = fd2d.habc_masks(120, 130, 50, multiple)
        for x, y in zip(a, b):
            if y is None:
                assert x is None
            else:
                assert np.array_equal(x.numpy(), y)


def test_config_reader_handles_template_subset():
    from seistorch_gb300.config import loads
    text = """
# comment
dtype: float32
equation: acoustic
geom:
  dt: 0.001
  h: 10.0
  multiple: false
  boundary:
    type: pml
    width: 50
  source_type:
    - h1
  invlist:
    vp: true
    rho: false
  wavelet:
  multiscale:
    - - 1.0
      - 3.0
    - 5.0
    - all
  shape: [3, 4]
"""
    c = loads(text)
    assert c["dtype"] == "float32" and c["geom"]["dt"] == 0.001
    assert c["geom"]["boundary"] == {"type": "pml", "width": 50}
    assert c["geom"]["source_type"] == ["h1"]
    assert c["geom"]["invlist"] == {"vp": True, "rho": False}
    assert c["geom"]["wavelet"] is None
    assert c["geom"]["multiscale"] == [[1.0, 3.0], 5.0, "all"]
    assert c["geom"]["shape"] == [3, 4]


def test_ricker_matches_oracle():
    from oracle import fd2d
    from seistorch_gb300.utils import ricker_wave
    assert np.array_equal(ricker_wave(12.0, 0.0005, 300, delay=90, dtype="numpy"),
                          fd2d.ricker(12.0, 0.0005, 300, delay=90))


def test_product_path_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "seistorch_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith(".py"):
                text = open(os.path.join(dirpath, fn)).read()
                assert "import oracle" not in text and "from oracle" not in text, fn


def test_gpu_entry_points_fail_loudly_without_cuda():
    from seistorch_gb300 import engine
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        engine.require_cuda(None, "x")


def test_elastic_io_maps_config_names_to_fields():
    from seistorch_gb300 import elastic_engine
    io, nch = elastic_engine.make_io(["txx", "tzz"], ["vx", "vz"])
    assert io.src_fields == (1 << 2) | (1 << 3) and nch == 2
    assert list(io.rec_fields)[:2] == [0, 1] and io.illum_field == 3
    io, nch = elastic_engine.make_io(["vz"], ["txz"])
    assert io.src_fields == 2 and list(io.rec_fields)[:1] == [4] and nch == 1
    with pytest.raises(ValueError):
        elastic_engine.make_io(["h1"], ["vx"])
    with pytest.raises(ValueError):
        elastic_engine.make_io(["txx"], ["vx", "vz", "txx", "tzz", "txz"])


def test_elastic_calls_validate_before_touching_the_gpu(lib):
    from seistorch_gb300 import _native as N
    g = N.Grid(64, 64, 64, 1, 0.0005, 5.0)
    fields = N.PTR5(*([16] * 5))
    assert lib.sgb_elastic_step(ctypes.byref(g), None, fields, fields, None) == 1
    m = N.ElasticModel(0, ctypes.c_void_p(20))
    assert lib.sgb_elastic_step(ctypes.byref(g), ctypes.byref(m), fields, fields, None) == 3
    m = N.ElasticModel(0, ctypes.c_void_p(16))
    assert lib.sgb_elastic_step(ctypes.byref(g), ctypes.byref(m), N.PTR5(16, 16, 0, 16, 16), fields, None) == 1
    bad = N.Grid(64, 66, 66, 1, 0.0005, 5.0)
    assert lib.sgb_elastic_step(ctypes.byref(bad), ctypes.byref(m), fields, fields, None) == 3
    io = N.ElasticIO(1 << 5, (ctypes.c_int32 * 4)(0, 1, 0, 0), 0)
    q = N.Acquisition()
    q.nt = 10
    cur = ctypes.c_int32(0)
    assert lib.sgb_elastic_forward(ctypes.byref(g), ctypes.byref(m), ctypes.byref(q), ctypes.byref(io),
                                   N.PTR10(*([16] * 10)), None, None, ctypes.byref(cur), None) == 1


def test_pickled_geometry_and_shot_files_round_trip(tmp_path):
    """Geometry in the reference's pickle layout (io.py:352-364) feeds
    setup_acquisition; shot gathers round-trip through the shot file."""
    from seistorch_gb300.io import SeisIO
    io = SeisIO()
    src = [[10, 2], [30, 2]]
    rec = [[list(range(0, 40)), [2] * 40]] * 2
    sp, rp = str(tmp_path / "src.pkl"), str(tmp_path / "rec.pkl")
    io.write_pkl(sp, src)
    io.write_pkl(rp, rec)
    cfg = {"geom": {"sources": sp, "receivers": rp}}
    s2, r2 = io.read_geom(cfg)
    assert s2 == src and r2 == rec
    with pytest.raises(FileNotFoundError):
        io.read_geom({"geom": {"sources": sp + "x", "receivers": rp}})
    shots = [np.random.default_rng(i).standard_normal((20, 40, 1)).astype(np.float32) for i in range(2)]
    path = io.write_shots(str(tmp_path / "obs.hdf5"), shots)
    for i in range(2):
        assert np.array_equal(io.read_shot(path, i), shots[i])


def test_vti_coefficient_map_matches_oracle():
    """engine.vti_coefficients (the planes the VTI kernels and their chain
    rule use) against the oracle's restatement of vti_habc2.py:36-51."""
    from oracle import fd2d
    from seistorch_gb300 import engine
    g = load("vti_habc2")
    vp, eps, delta = (g["models"][n] for n in ("vp", "epsilon", "delta"))
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    cx, cz = engine.vti_coefficients(t(vp), t(eps), t(delta), g["dt"], g["h"])
    sk = fd2d.vti_sk(eps, delta, g["h"])
    v2 = vp ** 2 * g["dt"] ** 2 / g["h"] ** 2
    assert rel_l2(cx.numpy(), v2 * (1 + 2 * eps + sk)) < 1e-14
    assert rel_l2(cz.numpy(), v2 * (1 + sk)) < 1e-14
    assert np.abs(sk[0]).max() == 0 and np.abs(sk[:, 0]).max() == 0  # zero frequency rows / columns


def test_rho_coefficient_map_zero_padding():
    """engine.rho_coefficients: C = dt^2 rho vp^2 / h^2 and the buoyancy
    averages with zeros beyond the grid (acoustic_rho_habc.py:44-51)."""
    from seistorch_gb300 import engine
    rng = np.random.default_rng(0)
    vp = 1500 + 1000 * rng.random((5, 6))
    rho = 1000 + 1500 * rng.random((5, 6))
    C, bxp, bxn, bzp, bzn = (p.numpy() for p in engine.rho_coefficients(torch.tensor(vp), torch.tensor(rho),
                                                                         0.001, 10.0))
    b = 1 / rho
    assert np.allclose(C, 1e-8 * rho * vp ** 2, rtol=1e-14)
    assert np.allclose(bxp[:, :-1], (b[:, :-1] + b[:, 1:]) / 2) and np.allclose(bxp[:, -1], b[:, -1] / 2)
    assert np.allclose(bxn[:, 1:], (b[:, :-1] + b[:, 1:]) / 2) and np.allclose(bxn[:, 0], b[:, 0] / 2)
    assert np.allclose(bzp[:-1], (b[:-1] + b[1:]) / 2) and np.allclose(bzp[-1], b[-1] / 2)
    assert np.allclose(bzn[1:], (b[:-1] + b[1:]) / 2) and np.allclose(bzn[0], b[0] / 2)


def test_neighbour_equation_entry_points_validate(lib):
    """The Born, VTI and variable-density entry points refuse a PML model or a
    missing plane before any CUDA call."""
    from seistorch_gb300 import _native as N
    g = N.Grid(64, 64, 64, 1, 0.001, 10.0)
    pml = N.AcousticModel(2, 0, 50, 0, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16))
    habc4 = N.AcousticModel(4, 1, 50, 0, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16))
    p = ctypes.c_void_p(16)
    assert lib.sgb_born_step(ctypes.byref(g), ctypes.byref(pml), p, p, p, p, p, p, p, p, None) == 5
    assert lib.sgb_vti_step(ctypes.byref(g), ctypes.byref(pml), p, p, p, None) == 5
    assert lib.sgb_vti_step(ctypes.byref(g), ctypes.byref(habc4), p, p, p, None) == 5  # 2nd order only
    assert lib.sgb_rho_step(ctypes.byref(g), ctypes.byref(habc4), p, p, p, p, None) == 5
    habc2 = N.AcousticModel(2, 1, 50, 0, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16))
    assert lib.sgb_rho_step(ctypes.byref(g), ctypes.byref(habc2), None, p, p, p, None) == 1
    assert lib.sgb_rho_step(ctypes.byref(g), ctypes.byref(habc2), ctypes.c_void_p(20), p, p, ctypes.c_void_p(32),
                            None) == 3


def test_born_loop_refuses_a_velocity_gradient():
    from seistorch_gb300 import engine
    vp = torch.ones(4, 4, requires_grad=True)
    with pytest.raises(NotImplementedError):
        engine.born_loop(vp, torch.zeros(4, 4), None, None, None)


def test_every_registered_equation_has_the_reference_entry_points():
    """build_model loads seistorch_gb300.equations2d.<equation> and needs its
    _time_step / _time_step_backward(_multiple) (model.py:64-80); the
    registry's parameter and wavefield lists name the same equations."""
    import importlib
    from seistorch_gb300.eqconfigure import Parameters, Wavefield
    paras = Parameters.valid_model_paras()
    for eq in paras:
        mod = importlib.import_module(f"seistorch_gb300.equations2d.{eq}")
        for fn in ("_time_step", "_time_step_backward", "_time_step_backward_multiple"):
            assert callable(getattr(mod, fn, None)), (eq, fn)
        assert Wavefield(eq).wavefields, eq
    for eq in Parameters.secondorder_equations():
        assert eq in paras and len(Wavefield(eq).wavefields) in (2, 4), eq
    assert paras["acoustic_lsrtm_habc"] == ["vp", "m"]
    assert Wavefield("vti_habc2").wavefields == ["p1", "p2"]


def test_cfl_check_limits_and_refusal(lib):
    """sgb_cfl_check: the leapfrog limit 2/sqrt(max eig(-h^2 L)) per order,
    1/sqrt(2) for the staggered elastic grid, and SGB_ERR_CFL above it
    (host only).  The workloads' Courant numbers (about 0.38 for 128x256 at
    4th order, 0.45 for 400x1000 at 8th order, 0.5 for the elastic 300x800
    grid) sit below their limits."""
    from seistorch_gb300 import _native as N
    want = {2: 1 / np.sqrt(2), 4: 1 / np.sqrt(8 / 3), 6: 1 / np.sqrt(2 * (1.5 + 1 / 90)),
            8: 1 / np.sqrt(2 * (8 / 5 + 8 / 315))}
    for order, lim in want.items():
        c, got = N.cfl_check(N.SCHEME_ACOUSTIC, order, 1000.0, 0.001, 10.0)
        assert abs(got - lim) < 1e-5 and abs(c - 0.1) < 1e-6
    assert abs(N.cfl_check(N.SCHEME_ELASTIC, 2, 1000.0, 0.0005, 5.0)[1] - 1 / np.sqrt(2)) < 1e-6
    assert N.cfl_check(N.SCHEME_ACOUSTIC, 4, 3800.0, 0.001, 10.0)[0] < want[4]
    assert N.cfl_check(N.SCHEME_ACOUSTIC, 8, 4500.0, 0.001, 10.0)[0] < want[8]
    assert N.cfl_check(N.SCHEME_ELASTIC, 2, 5000.0, 0.0005, 5.0)[0] < 1 / np.sqrt(2)
    # a bad dt: 4500 m/s at 10 m needs dt below 1.23 ms at 8th order
    with pytest.raises(N.NativeError, match="CFL"):
        N.cfl_check(N.SCHEME_ACOUSTIC, 8, 4500.0, 0.0013, 10.0)
    with pytest.raises(N.NativeError, match="CFL"):
        N.cfl_check(N.SCHEME_ELASTIC, 2, 5000.0, 0.0008, 5.0)
    out = ctypes.c_float(0.0)
    assert lib.sgb_cfl_check(0, 2, 2000.0, 0.004, 10.0, ctypes.byref(out), None) == 9
    assert abs(out.value - 0.8) < 1e-6
    assert lib.sgb_status_string(9).startswith(b"CFL")
    assert lib.sgb_cfl_check(0, 3, 2000.0, 0.001, 10.0, None, None) == 5   # order
    assert lib.sgb_cfl_check(1, 4, 2000.0, 0.001, 10.0, None, None) == 5   # elastic is 2nd order
    assert lib.sgb_cfl_check(0, 2, 2000.0, -0.001, 10.0, None, None) == 1  # dt
    assert lib.sgb_cfl_check(2, 2, 2000.0, 0.001, 10.0, None, None) == 1   # scheme


def test_cfl_limit_is_the_stencil_stability_edge():
    """The acoustic limit is where the leapfrog recursion's amplification at
    the worst wavenumber reaches 1: just below it a plane wave of that
    wavenumber stays bounded over many steps, just above it it grows."""
    from oracle import fd2d
    from seistorch_gb300 import _native as N
    for order in (2, 4, 8):
        lim = N.cfl_check(N.SCHEME_ACOUSTIC, order, 0.1, 1.0, 1.0)[1]
        c = fd2d.fd_coefficients(order)
        th = np.linspace(0, np.pi, 4097)
        s1 = np.max(2 * sum(cj * (1 - np.cos((j + 1) * th)) for j, cj in enumerate(c)))
        for fac, bounded in ((0.999, True), (1.001, False)):
            a = (fac * lim) ** 2 * 2 * s1  # C^2 * max eig of -h^2 L
            u0, u1 = 1.0, 1.0
            for _ in range(20000):
                u0, u1 = u1, (2 - a) * u1 - u0
            assert (abs(u1) < 1e3) == bounded, (order, fac, u1)


@pytest.mark.parametrize("name", ["acoustic_habc_o2", "acoustic_habc_o2_multiple", "elastic"])
def test_save_restore_boundaries_match_reference(name):
    """save_boundaries / restore_boundaries (equations2d/utils.py:50-90) on
    the fields the step goldens hold: the strips the reference saved from
    one state, and the reference's restore of another state's strips into
    it (with and without ``multiple``)."""
    from seistorch_gb300.equations2d.utils import restore_boundaries, save_boundaries
    z = np.load(os.path.join(ROOT, "tests", "golden", f"steps_{name}.npz"))
    f0 = str(z["field_names"][0])
    tgt = torch.tensor(z["restore_target"], dtype=torch.float64)
    for got, k in zip(save_boundaries(tgt), "tblr"):
        assert np.array_equal(got.numpy(), z[f"strip_{f0}_{k}"].astype(np.float64))
    strips = save_boundaries(torch.tensor(z["in_" + f0], dtype=torch.float64))
    assert np.array_equal(restore_boundaries(tgt.clone(), strips).numpy(), z["restored"].astype(np.float64))
    assert np.array_equal(restore_boundaries(tgt.clone(), strips, multiple=True).numpy(),
                          z["restored_multiple"].astype(np.float64))


def test_diff_using_roll_edge_rule():
    """Only dim 1 and dim 2 (the last axis) get the padding value at the
    wrapped edge (equations2d/utils.py:17-23,37-43); other dims keep the wrap."""
    from seistorch_gb300.equations2d.utils import diff_using_roll
    x = torch.arange(24.0).reshape(2, 3, 4) ** 2
    f1 = diff_using_roll(x, 1)
    assert torch.all(f1[:, 0] == 0) and torch.equal(f1[:, 1:], x[:, 1:] - x[:, :-1])
    b2 = diff_using_roll(x, 2, False)
    assert torch.all(b2[..., -1] == 0) and torch.equal(b2[..., :-1], x[..., 1:] - x[..., :-1])
    wrap = diff_using_roll(x, -1)  # not 1 or 2: the roll's wrap stays
    assert torch.equal(wrap, x - torch.roll(x, 1, -1))


def test_hdf5_shot_gathers_round_trip(tmp_path):
    """HDF5 shot gathers in the reference's layout (io.py:97-115): one float32
    dataset ``shot_<i>`` of shape (nt, nrec, nch) per shot.  A file written
    the way the reference's ``create_hdf5_file`` + per-shot writes lay it out
    reads back through ``SeisIO.read_shot``, and ``SeisIO.write_shots``
    produces that layout.  Runs wherever h5py is installed."""
    h5py = pytest.importorskip("h5py")
    from seistorch_gb300.io import SeisIO
    rng = np.random.default_rng(0)
    shots = [rng.standard_normal((50, 7 + i, 2)).astype(np.float32) for i in range(3)]
    ref_path = str(tmp_path / "ref.hdf5")
    with h5py.File(ref_path, "w") as f:
        for i, s in enumerate(shots):
            f.create_dataset(f"shot_{i}", s.shape, dtype="f", chunks=True)
            f[f"shot_{i}"][...] = s
    for i, s in enumerate(shots):
        assert np.array_equal(SeisIO.read_shot(ref_path, i), s)
    out = SeisIO.write_shots(str(tmp_path / "ours.hdf5"), shots)
    with h5py.File(out, "r") as f:
        assert sorted(f.keys()) == ["shot_0", "shot_1", "shot_2"]
        for i, s in enumerate(shots):
            assert f[f"shot_{i}"].dtype == np.float32
            assert np.array_equal(f[f"shot_{i}"][...], s)
