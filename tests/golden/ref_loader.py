"""Load the reference seistorch hot-path modules on a CPU-only machine.

Golden-fixture generation only: this module imports the reference source tree
(``REF_ROOT``) in-process, so it runs only where that tree exists.  Nothing in
the product, the GPU tests, ``smoke()`` or ``bench.py`` imports it.

The reference package ``seistorch/__init__.py`` pulls in optional third-party
modules (yaml, h5py, geomloss, torchvision, torchaudio, segyio, obspy,
tensorboard, prettytable, ...).  Those are absent here, so this loader:

* registers a bare ``seistorch`` package whose ``__path__`` is the reference
  package directory (so ``__init__`` never runs),
* registers empty stub modules for the missing third-party names,
* execs ``equations2d/acoustic.py``, ``acoustic_habc.py``,
  ``acoustic_lsrtm_habc.py`` and ``vacoustic_habc.py`` from source with their
  module-level ``device = "cuda"`` (acoustic.py:56, acoustic_habc.py:57,
  acoustic_lsrtm_habc.py:7, vacoustic_habc.py:57) replaced by ``"cpu"`` so the FD kernel can be built
  without a GPU, and lets the caller patch ``spatial_order``/``kernel``
  (module globals read at call time, acoustic.py:55-58).
"""
import importlib
import importlib.util
import os
import sys
import types

# the reference checkout must be named explicitly (no machine-specific default)
REF_ROOT = os.environ.get("SEISTORCH_REF_ROOT", "")
PKG_DIR = os.path.join(REF_ROOT, "seistorch")

_STUB_ROOTS = ["yaml", "h5py", "geomloss", "torchvision", "torchaudio", "segyio",
               "obspy", "tensorboard", "prettytable", "setproctitle", "ot",
               "mpi4py", "matplotlib", "numba", "pywt", "cv2", "skimage"]


class _StubModule(types.ModuleType):
    def __getattr__(self, attr):
        if attr.startswith("__"):
            raise AttributeError(attr)
        # any attribute access yields a harmless placeholder class
        return type(attr, (), {"__init__": lambda self, *a, **k: None})


class _StubFinder:
    """Meta-path finder that serves an empty module for any missing name
    under one of ``_STUB_ROOTS`` (e.g. ``torchvision.transforms.functional``)."""

    def find_spec(self, fullname, path=None, target=None):
        root = fullname.split(".")[0]
        if root not in _STUB_ROOTS:
            return None
        return importlib.util.spec_from_loader(fullname, self, is_package=True)

    def create_module(self, spec):
        mod = _StubModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        pass


def _install_stubs():
    for root in list(_STUB_ROOTS):
        try:
            importlib.import_module(root)
        except Exception:
            continue
        # importable for real: never stub it
        _STUB_ROOTS.remove(root)
    if not any(isinstance(f, _StubFinder) for f in sys.meta_path):
        sys.meta_path.append(_StubFinder())
    tb = "torch.utils.tensorboard"
    if tb not in sys.modules:
        try:
            importlib.import_module(tb)
        except Exception:
            mod = _StubModule(tb)
            mod.__path__ = []
            sys.modules[tb] = mod


def _install_package():
    if "seistorch" in sys.modules and getattr(sys.modules["seistorch"], "_graft_stub", False):
        return
    pkg = types.ModuleType("seistorch")
    pkg.__path__ = [PKG_DIR]
    pkg._graft_stub = True
    sys.modules["seistorch"] = pkg
    sub = types.ModuleType("seistorch.equations2d")
    sub.__path__ = [os.path.join(PKG_DIR, "equations2d")]
    sys.modules["seistorch.equations2d"] = sub


def _exec_patched(modname, path, device, line_patches=()):
    with open(path) as f:
        src = f.read()
    for old, new in line_patches:
        src = src.replace(old, new)
    src = src.replace('device = "cuda"', f'device = "{device}"')
    spec = importlib.util.spec_from_loader(modname, loader=None, origin=path)
    mod = importlib.util.module_from_spec(spec)
    mod.__file__ = path
    mod.__package__ = modname.rpartition(".")[0]
    sys.modules[modname] = mod
    exec(compile(src, path, "exec"), mod.__dict__)
    return mod


def load(device="cpu"):
    """Return a namespace with the reference hot-path modules."""
    if not REF_ROOT or not os.path.isdir(PKG_DIR):
        raise RuntimeError("set SEISTORCH_REF_ROOT to a seistorch checkout (the directory holding seistorch/)")
    _install_stubs()
    _install_package()
    ns = types.SimpleNamespace()
    ns.utils2d = importlib.import_module("seistorch.equations2d.utils")
    ns.acoustic = _exec_patched("seistorch.equations2d.acoustic",
                                os.path.join(PKG_DIR, "equations2d", "acoustic.py"), device)
    ns.acoustic_habc = _exec_patched("seistorch.equations2d.acoustic_habc",
                                     os.path.join(PKG_DIR, "equations2d", "acoustic_habc.py"), device)
    ns.acoustic_lsrtm_habc = _exec_patched("seistorch.equations2d.acoustic_lsrtm_habc",
                                           os.path.join(PKG_DIR, "equations2d", "acoustic_lsrtm_habc.py"), device)
    # convkernel.py:71 picks "cuda" or an Exception object as its device
    ns.convkernel = _exec_patched(
        "seistorch.equations2d.convkernel", os.path.join(PKG_DIR, "equations2d", "convkernel.py"), device,
        [('device = "cuda" if torch.cuda.is_available() else Exception("No cuda device found")',
          f'device = "{device}"')])
    ns.vacoustic_habc = _exec_patched("seistorch.equations2d.vacoustic_habc",
                                      os.path.join(PKG_DIR, "equations2d", "vacoustic_habc.py"), device)
    ns.vti_habc2 = importlib.import_module("seistorch.equations2d.vti_habc2")
    ns.acoustic_rho_habc = importlib.import_module("seistorch.equations2d.acoustic_rho_habc")
    ns.elastic = importlib.import_module("seistorch.equations2d.elastic")
    ns.pml = importlib.import_module("seistorch.pml")
    ns.habc = importlib.import_module("seistorch.habc")
    ns.eqconfigure = importlib.import_module("seistorch.eqconfigure")
    ns.source = importlib.import_module("seistorch.source")
    ns.probe = importlib.import_module("seistorch.probe")
    ns.cell = importlib.import_module("seistorch.cell")
    ns.checkpoint = importlib.import_module("seistorch.checkpoint")
    ns.checkpoint_new = importlib.import_module("seistorch.checkpoint_new")
    ns.rnn = importlib.import_module("seistorch.rnn")
    ns.rutils = importlib.import_module("seistorch.utils")
    ns.type = importlib.import_module("seistorch.type")
    return ns


def set_spatial_order(mod, order, dtype=None):
    """Patch the module-level FD kernel of acoustic(.py|_habc.py) to `order`."""
    import torch
    k = mod.generate_convolution_kernel(order).unsqueeze(0).unsqueeze(0)
    if dtype is not None:
        k = k.to(dtype)
    mod.spatial_order = order
    mod.kernel = k.to(mod.device)
    mod.padding = mod.kernel.shape[-1] // 2


def make_geom(ref, equation, models, d, dt, h, *, use_habc=False, bwidth=50,
              multiple=False, source_type=("h1",), receiver_type=("h1",),
              inversion=False, boundary_saving=False, requires_grad=(),
              source_illumination=False, dtype=None):
    """Build a stand-in for ``WaveGeometryFreeForm`` (geom.py:97-240).

    `models` maps parameter names (eqconfigure.py:8-28 order) to padded
    (Nz, Nx) arrays.  Only the attributes that ``WaveCell``/``WaveRNN``
    read (cell.py:12-77, rnn.py:14-217) are provided.
    """
    import torch
    dtype = dtype or torch.get_default_dtype()

    class _Geom(torch.nn.Module):
        pass

    g = _Geom()
    names = ref.eqconfigure.Parameters.valid_model_paras()[equation]
    first = None
    for n in names:
        arr = torch.as_tensor(models[n], dtype=dtype)
        first = arr if first is None else first
        g.register_parameter(n, torch.nn.Parameter(arr.clone(), requires_grad=n in requires_grad))
    g.register_buffer("h", torch.tensor(float(h), dtype=dtype))
    g.register_buffer("_d", torch.as_tensor(d, dtype=dtype).clone())
    g.d = g._d
    g.dt = float(dt)
    g.domain_shape = tuple(first.shape)
    g.equation = equation
    g.use_habc = use_habc
    g.bwidth = bwidth
    g.multiple = multiple
    g.device = "cpu"
    g.boundary_saving = boundary_saving
    g.inversion = inversion
    g.use_implicit = False
    g.source_illumination = source_illumination
    g.model_parameters = list(names)
    g.source_type = list(source_type)
    g.receiver_type = list(receiver_type)
    return g


def run_wavernn(ref, geom, fwd, bwd, wavelet, src_zx, rec_zx):
    """Run the reference ``WaveRNN.forward`` (rnn.py:100-217).

    src_zx: list of (z, x) per shot (padded grid indices);
    rec_zx: list per shot of (zs, xs) lists.  Returns the ``WaveRNN``
    module and its TensorList of per-shot records (nt, nrec, nch).
    """
    import torch
    cell = ref.cell.WaveCell(geom, fwd, bwd)
    rnn = ref.rnn.WaveRNN(cell, source_encoding=False)
    sources = [ref.source.WaveSource(x=int(x), y=int(z)) for (z, x) in src_zx]
    probes = [ref.probe.WaveIntensityProbe(x=list(map(int, xs)), y=list(map(int, zs)))
              for (zs, xs) in rec_zx]
    rnn.reset_sources(sources)
    rnn.reset_probes(probes)
    x = torch.as_tensor(wavelet, dtype=torch.get_default_dtype()).reshape(1, -1)
    y = rnn(x)
    return rnn, y
