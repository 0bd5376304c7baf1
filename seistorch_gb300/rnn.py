"""Time loop (seistorch/rnn.py:14-217) dispatched to the native engine.

``WaveRNN.forward(x, omega, super_source, super_probes, vp)`` has the
reference signature and returns the same ``TensorList`` of per-shot records
(nt, nrec, nch).  The whole loop -- step, source injection, receiver
sampling, illumination -- is one C-ABI call; when a model parameter requires
grad, the loop is a differentiable op whose backward is the fused
boundary-saving adjoint kernel.
"""
from typing import Iterator, Tuple

import torch
from torch.nn.parameter import Parameter

from . import engine
from .acquisition import merge_receivers_with_same_keys, merge_sources_with_same_keys
from .acquisition import setup_acquisition
from .eqconfigure import Parameters, Wavefield
from .probe import WaveProbe
from .source import WaveSource
from .type import TensorList


class WaveRNN(torch.nn.Module):
    def __init__(self, cell, source_encoding=False):
        super().__init__()
        self.cell = cell
        self.source_encoding = source_encoding
        self.use_implicit = False
        self.second_order_equation = self.cell.geom.equation in Parameters.secondorder_equations()
        self.source_illumination = self.cell.geom.source_illumination
        self.sources = torch.nn.ModuleList()
        self.probes = torch.nn.ModuleList()

    def named_parameters(self, prefix: str = "", recurse: bool = True,
                         remove_duplicate: bool = True) -> Iterator[Tuple[str, Parameter]]:
        yield from self.cell.geom.named_parameters(prefix, recurse, remove_duplicate)

    def reset_sources(self, sources):
        self.sources = torch.nn.ModuleList(sources if isinstance(sources, list) else [sources])

    def reset_probes(self, probes):
        self.probes = torch.nn.ModuleList(probes if isinstance(probes, list) else [probes])

    def reset_geom(self, shots, src_list, rec_list, cfg):
        sources, receivers = setup_acquisition(shots, src_list, rec_list, cfg)
        self.reset_sources(sources)
        self.reset_probes(receivers)

    def _acquisition(self, x, super_source, super_probes, nz, nx, device):
        # The device tables of the batch's sources and receivers are rebuilt
        # only when the geometry changes: the key holds every source / probe
        # module's buffers (storage, in-place version, shape), so reset_geom
        # or an in-place edit of a coordinate invalidates it; a hit is a
        # copy with this call's wavelet.
        key = None
        if super_source is None and super_probes is None:
            key = (nz, nx, int(x.shape[0]), bool(self.source_encoding), str(device)) + tuple(
                (id(m), name, buf.data_ptr(), buf._version, tuple(buf.shape))
                for m in list(self.sources) + list(self.probes) for name, buf in m.named_buffers())
            hit = getattr(self, "_acq_cache", None)
            if hit is not None and hit[0] == key:
                return hit[1].with_wavelet(x), list(hit[2])
        if super_source is None:
            bidx_source, keys = merge_sources_with_same_keys(self.sources)
            super_source = WaveSource(bidx_source, self.second_order_equation, **keys)
        if super_probes is None:
            reccounts, bidx_rec, reckeys = merge_receivers_with_same_keys(self.probes)
            super_probes = WaveProbe(bidx_rec, **reckeys)
        else:
            reccounts = list(super_probes.reccounts)
        sx = super_source.x.reshape(-1).tolist()
        sy = super_source.y.reshape(-1).tolist()
        nw = x.shape[0]
        if self.source_encoding:
            sources = [[(z, xx) for z, xx in zip(sy, sx)]]
            wrows = [[i if nw > 1 else 0 for i in range(len(sx))]]
        else:
            sources = [[(z, xx)] for z, xx in zip(sy, sx)]
            wrows = [[b if nw == len(sx) and nw > 1 else 0] for b in range(len(sx))]
        nshots = len(sources)
        bidx = torch.as_tensor(super_probes.bidx).reshape(-1).cpu()
        py = super_probes.y.reshape(-1).cpu()
        px = super_probes.x.reshape(-1).cpu()
        receivers = []
        for b in range(nshots):
            sel = bidx == b
            receivers.append((py[sel].tolist(), px[sel].tolist()))
        if sum(len(r[0]) for r in receivers) != sum(reccounts):
            raise ValueError("receivers refer to shots outside the batch")
        acq = engine.Acquisition(nz, nx, sources, receivers, x, device, src_wrow=wrows)
        if key is not None:
            self._acq_cache = (key, acq, reccounts)
        return acq, reccounts

    def forward(self, x, omega=10.0, super_source=None, super_probes=None, vp=None):
        geom = self.cell.geom
        models = [getattr(geom, n) for n in geom.model_parameters]
        if vp is not None:
            models[0] = vp
        device = models[0].device
        engine.require_cuda(models[0], "WaveRNN.forward")
        nz, nx = geom.domain_shape
        x = torch.as_tensor(x).to(device=device, dtype=torch.float32)
        if x.ndim == 1:
            x = x[None]
        acq, reccounts = self._acquisition(x, super_source, super_probes, nz, nx, device)
        eq = geom.equation
        d = geom.d.to(device)
        illum = None
        if eq in ("acoustic", "acoustic_habc"):
            if list(geom.source_type) != ["h1"] or list(geom.receiver_type) != ["h1"]:
                raise NotImplementedError("acoustic equations inject into and record h1")
            prop = engine.AcousticPropagator(nz, nx, geom.dt, float(geom.h), geom.spatial_order,
                                             "habc" if geom.use_habc else "pml", geom.bwidth,
                                             geom.multiple, device)
            ck = geom.ckpt_every or engine.default_ckpt_every(acq.nt)
            rec, illum = engine.acoustic_loop(models[0].to(torch.float32), prop, d, acq,
                                              self.source_illumination, ck)
            self._fields = prop
        elif eq == "acoustic_lsrtm_habc":
            if list(geom.source_type) != ["h1"] or list(geom.receiver_type) != ["sh1"]:
                raise NotImplementedError("Born modelling injects into h1 and records sh1")
            if not geom.use_habc:
                raise NotImplementedError("acoustic_lsrtm_habc runs with the HABC boundary")
            prop = engine.BornPropagator(nz, nx, geom.dt, float(geom.h), geom.spatial_order, geom.bwidth,
                                         geom.multiple, device)
            ck = geom.ckpt_every or engine.default_ckpt_every(acq.nt)
            rec = engine.born_loop(models[0].to(torch.float32), models[1].to(torch.float32), prop, d, acq, ck)
            self._fields = prop
        elif eq == "acoustic_rho_habc":
            if list(geom.source_type) != ["h1"] or list(geom.receiver_type) != ["h1"]:
                raise NotImplementedError("acoustic_rho_habc injects into and records h1")
            if not geom.use_habc:
                raise NotImplementedError("acoustic_rho_habc runs with the HABC boundary")
            prop = engine.RhoPropagator(nz, nx, geom.dt, float(geom.h), geom.bwidth, geom.multiple, device)
            ck = geom.ckpt_every or engine.default_ckpt_every(acq.nt)
            rec = engine.rho_loop(models[0].to(torch.float32), models[1].to(torch.float32), prop, d, acq, ck)
            self._fields = prop
        elif eq == "vti_habc2":
            if list(geom.source_type) != ["p1"] or list(geom.receiver_type) != ["p1"]:
                raise NotImplementedError("vti_habc2 injects into and records p1")
            if not geom.use_habc:
                raise NotImplementedError("vti_habc2 runs with the HABC boundary")
            prop = engine.VTIPropagator(nz, nx, geom.dt, float(geom.h), geom.bwidth, geom.multiple, device)
            ck = geom.ckpt_every or engine.default_ckpt_every(acq.nt)
            rec = engine.vti_loop(*[m_.to(torch.float32) for m_ in models[:3]], prop, d, acq, ck)
            self._fields = prop
        elif eq == "vacoustic_habc":
            if list(geom.source_type) != ["h1"] or list(geom.receiver_type) != ["h1"]:
                raise NotImplementedError("vacoustic_habc injects into and records h1")
            if not geom.use_habc:
                raise NotImplementedError("vacoustic_habc runs with the HABC boundary")
            prop = engine.VacousticPropagator(nz, nx, geom.dt, float(geom.h), geom.spatial_order, geom.bwidth,
                                              geom.multiple, device)
            rec = engine.vacoustic_records(models[0].to(torch.float32), models[1].to(torch.float32), prop, d, acq)
            self._fields = prop
        elif eq == "elastic":
            from . import elastic_engine
            rec, illum, fields = elastic_engine.elastic_loop(models, geom, d, acq,
                                                             self.source_illumination)
        else:
            raise NotImplementedError(f"equation '{eq}' is not implemented by seistorch_gb300")
        if self.source_illumination:
            self.precondition = illum
        y = TensorList(torch.split(rec, reccounts, dim=1))
        y.has_nan()
        return y
