"""Model geometry (seistorch/geom.py:15-240): grid spacing, time step,
boundary coefficients and the edge-padded model parameters."""
import numpy as np
import torch

from .eqconfigure import Parameters
from .habc import generate_habc_coefficients_2d
from .pml import generate_pml_coefficients_2d


class WaveGeometryFreeForm(torch.nn.Module):
    """``WaveGeometryFreeForm(mode, logger, **cfg)``.

    Model arrays come from ``models={name: array}`` when given, else from the
    ``.npy`` files of ``cfg['VEL_PATH']``.  Each becomes an ``nn.Parameter``
    edge-padded by the boundary width (top unpadded with ``multiple``,
    geom.py:213-240), trainable when ``mode != 'forward'`` and ``invlist``
    says so.  ``geom.spatial_order`` (default 2, the reference's hard-wired
    order, acoustic.py:55) selects the acoustic stencil order.
    """

    def __init__(self, mode="forward", logger=None, models=None, **kwargs):
        super().__init__()
        g = kwargs["geom"]
        self.mode = mode
        self.kwargs = kwargs
        self.logger = logger
        self.unit = g.get("unit", 1.0) or 1.0
        self.dt = float(g["dt"])
        self.dh = float(g["h"]) * self.unit
        self.register_buffer("h", torch.tensor(self.dh))
        self.device = kwargs.get("device", "cuda")
        btype = g["boundary"]["type"]
        if btype not in ("pml", "habc"):
            raise ValueError("boundary type must be one of [pml, habc] in seistorch_gb300")
        self.bwidth = int(g["boundary"]["width"])
        self.use_pml = btype == "pml" and self.bwidth > 0
        self.use_habc = btype == "habc" and self.bwidth > 0
        self.use_random = False
        if self.use_habc:
            self.bwidth = 50  # fixed for HABC (geom.py:62-65)
        self.multiple = bool(g.get("multiple", False))
        self.boundary_saving = bool(g.get("boundary_saving", True))
        elastic = kwargs["equation"] == "elastic"
        self.source_type = list(g.get("source_type") or (["txx", "tzz"] if elastic else ["h1"]))
        self.receiver_type = list(g.get("receiver_type") or (["vx", "vz"] if elastic else ["h1"]))
        self.source_illumination = bool(g.get("source_illumination", False))
        self.spatial_order = int(g.get("spatial_order", 2))
        self.ckpt_every = int(g.get("ckpt_every", 0) or 0)
        self.equation = kwargs["equation"]
        self.use_implicit = False
        self.inversion = False
        self.ndim = 2
        self.model_parameters = []
        self.pars_need_invert = []
        invlist = g.get("invlist") or {}
        paths = kwargs.get("VEL_PATH") or {}
        for name in Parameters.valid_model_paras()[self.equation]:
            if models is not None and name in models:
                arr = np.asarray(models[name], dtype=np.float64)
            else:
                arr = np.load(paths[name])
            arr = arr * self.unit
            pad = np.pad(arr, self.padding_list, mode="edge")
            invert = bool(invlist.get(name, False)) and mode != "forward"
            if invert:
                self.pars_need_invert.append(name)
            self.model_parameters.append(name)
            self.register_parameter(name, torch.nn.Parameter(
                torch.as_tensor(pad, dtype=torch.get_default_dtype()), requires_grad=invert))
        self.domain_shape = tuple(getattr(self, self.model_parameters[0]).shape)
        if self.use_habc:
            d = generate_habc_coefficients_2d(self.domain_shape, self.bwidth, multiple=self.multiple)
        elif self.use_pml:
            d = generate_pml_coefficients_2d(self.domain_shape, self.bwidth, multiple=self.multiple)
        else:
            d = torch.zeros(self.domain_shape)
        self.register_buffer("_d", d.to(torch.get_default_dtype()))

    @property
    def padding_list(self):
        top = 0 if self.multiple else self.bwidth
        return [[top, self.bwidth], [self.bwidth, self.bwidth]]

    @property
    def d(self):
        return self._d

    def forward(self):
        raise NotImplementedError("WaveGeometry only holds parameters")
