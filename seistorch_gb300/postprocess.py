"""Misfit and gradient post-processing on the device, with seistorch's names.

``filter_records`` (SeisSignal.filter, signal.py:39-101): Butterworth
low-/band-pass applied forward and backward (zero phase) to every trace.
``L2`` (loss.py:409-421): sum over shots of MSELoss(reduction='sum'); its
backward is the adjoint source 2 (syn - obs) from the same kernel pass.
``precondition`` / ``cut_gradient`` (process.py:43-47, 115-118),
``smooth_gradient`` (process.py:66-113 with signal.gaussian_filter,
signal.py:247-319) and ``Steepestdescent`` (optimizer.py:124-142) run the
kernels of ``postproc.cu``.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .engine import pitch_of, require_cuda, to_pitched


class _L2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, syn, obs):
        require_cuda(syn, "L2")
        syn_c = syn.contiguous().to(torch.float32)
        obs_c = obs.contiguous().to(torch.float32).to(syn.device)
        resid = torch.empty_like(syn_c)
        loss = torch.zeros(1, dtype=torch.float64, device=syn.device)
        N.call("sgb_l2_misfit", syn_c.numel(), N.ptr(syn_c), N.ptr(obs_c), N.ptr(resid), N.ptr(loss),
               N.stream_handle())
        ctx.save_for_backward(resid)
        return loss[0].to(syn.dtype)

    @staticmethod
    def backward(ctx, g):
        (resid,) = ctx.saved_tensors
        return resid * g.to(resid.dtype), None


class L2(torch.nn.Module):
    """``L2()(x, y)`` for lists of per-shot records (or two tensors)."""

    @property
    def name(self):
        return "l2"

    def forward(self, x, y):
        if isinstance(x, torch.Tensor):
            return _L2.apply(x, y)
        loss = 0.0
        for a, b in zip(x, y):
            loss = loss + _L2.apply(a, b)
        return loss


def precondition(grad, illum=None, eps=0.0, mask=None):
    """grad (* mask) / (illum + eps) on the device (eps = 0: the reference)."""
    require_cuda(grad, "precondition")
    nz, nx = grad.shape
    p = pitch_of(nx)
    g = to_pitched(grad.detach(), p).contiguous()
    il = to_pitched(illum.detach(), p).contiguous() if illum is not None else None
    mk = to_pitched(mask.to(grad.device), p).contiguous() if mask is not None else None
    out = torch.empty_like(g)
    N.call("sgb_grad_precondition", nz, nx, p, N.ptr(g), N.ptr(il), ctypes.c_float(eps), N.ptr(mk), N.ptr(out),
           N.stream_handle())
    return out[:, :nx]


def cut_gradient(grad, mask):
    return precondition(grad, None, 0.0, mask)


def gaussian_weights(sigma, radius):
    """Normalised taps of signal.gaussian_filter (kernel size 2 radius + 1).
    An odd radius gives the reference an even kernel and an output one
    sample longer than its input; it is rejected here."""
    if radius % 2 != 0:
        raise ValueError("smoothing radius must be even (an odd radius changes the array shape in the reference)")
    ks = 2 * radius + 1
    k = np.exp(-(np.arange(ks) - ks // 2) ** 2 / (2 * sigma ** 2))
    return (k / k.sum()).astype(np.float32)


def smooth_gradient(grad, sigma, radius, counts=1):
    """``counts`` passes along z then x; sigma / radius: dicts with 'z', 'x'."""
    require_cuda(grad, "smooth_gradient")
    nz, nx = grad.shape
    p = pitch_of(nx)
    g = to_pitched(grad.detach().to(torch.float32), p).contiguous().clone()
    tmp = torch.empty_like(g)
    wz = torch.tensor(gaussian_weights(sigma["z"], radius["z"]), device=grad.device)
    wx = torch.tensor(gaussian_weights(sigma["x"], radius["x"]), device=grad.device)
    N.call("sgb_grad_smooth", nz, nx, p, N.ptr(wz), radius["z"], N.ptr(wx), radius["x"], counts, N.ptr(g),
           N.ptr(tmp), N.stream_handle())
    return g[:, :nx]


class Steepestdescent(torch.optim.Optimizer):
    """param -= lr * d / max|d|, d = grad clamped to its 2 % / 98 % quantiles
    when ``grad_clamp`` (optimizer.py:124-142)."""

    name = "sd"

    def __init__(self, params, lr=10.0, grad_clamp=True, **kwargs):
        super().__init__(params, dict(lr=lr, grad_clamp=grad_clamp))
        self._scratch = {}

    @torch.no_grad()
    def step(self, closure=None):
        loss = closure() if closure is not None else None
        for group in self.param_groups:
            for p in group["params"]:
                if p.grad is None:
                    continue
                g = p.grad.contiguous().to(torch.float32)
                lo = hi = 0.0
                if group["grad_clamp"]:
                    q = torch.quantile(g.reshape(-1), torch.tensor([0.02, 0.98], device=g.device))
                    lo, hi = float(q[0]), float(q[1])
                s = self._scratch.get(p.device)
                if s is None:
                    s = self._scratch[p.device] = torch.zeros(1, dtype=torch.int32, device=p.device)
                if p.dtype != torch.float32 or not p.is_contiguous():
                    raise TypeError("Steepestdescent updates contiguous float32 parameters")
                N.call("sgb_sd_step", p.numel(), N.ptr(p), N.ptr(g), ctypes.c_float(group["lr"]),
                       int(group["grad_clamp"]), ctypes.c_float(lo), ctypes.c_float(hi), N.ptr(s),
                       N.stream_handle())
        return loss


class Cg(torch.optim.Optimizer):
    """Non-linear conjugate gradient (optimizer.py:144-224): d = grad clamped
    to its clip_value / 1 - clip_value quantiles when ``grad_clamp``; beta =
    Polak-Ribiere ('PR') or Fletcher-Reeves ('FR'), 0 on the first step;
    direction = -d + beta direction; param += lr direction / max|direction|.
    One native call per parameter (sgb_ncg_step), no host synchronisation
    besides the quantiles."""

    name = "ncg"

    def __init__(self, params, lr=1.0, beta_type="PR", grad_clamp=True, clip_value=0.02, **kwargs):
        if beta_type not in ("PR", "FR"):
            raise ValueError("Invalid beta_type. Must be 'FR' or 'PR'")
        super().__init__(params, dict(lr=lr, beta_type=beta_type, grad_clamp=grad_clamp, clip_value=clip_value))
        self._scratch = {}

    @torch.no_grad()
    def step(self, closure=None):
        loss = closure() if closure is not None else None
        for group in self.param_groups:
            for p in group["params"]:
                if p.grad is None:
                    continue
                if p.dtype != torch.float32 or not p.is_contiguous():
                    raise TypeError("Cg updates contiguous float32 parameters")
                g = p.grad.contiguous().to(torch.float32)
                lo = hi = 0.0
                if group["grad_clamp"]:
                    c = float(group["clip_value"])
                    q = torch.quantile(g.reshape(-1), torch.tensor([c, 1.0 - c], device=g.device))
                    lo, hi = float(q[0]), float(q[1])
                state = self.state[p]
                if len(state) == 0:
                    state["step"] = 0
                    state["prev_grad"] = torch.zeros_like(g)
                    state["direction"] = torch.zeros_like(g)
                s = self._scratch.get(p.device)
                if s is None:
                    s = self._scratch[p.device] = torch.zeros(4, dtype=torch.float64, device=p.device)
                N.call("sgb_ncg_step", p.numel(), N.ptr(p), N.ptr(g), N.ptr(state["prev_grad"]),
                       N.ptr(state["direction"]), ctypes.c_float(group["lr"]),
                       0 if group["beta_type"] == "PR" else 1, int(group["grad_clamp"]), ctypes.c_float(lo),
                       ctypes.c_float(hi), N.ptr(s), N.stream_handle())
                state["step"] += 1
        return loss


def filter_mode(freqs):
    """SeisSignal.decide_filter_type: a number or [f] -> lowpass, [f1, f2] -> bandpass."""
    if freqs == "all":
        return "all"
    if isinstance(freqs, (int, float)):
        return "lowpass"
    if isinstance(freqs, (list, tuple)):
        return "lowpass" if len(freqs) == 1 else "bandpass"
    raise ValueError(f"cannot filter with frequencies {freqs!r}")


def filter_records(records, dt, freqs, order=4):
    """Zero-phase Butterworth filter of records (nt, ntraces[, nch]) along time
    on the device; the filter is designed with scipy.signal.butter as the
    reference does (Wn = 2 f dt)."""
    from scipy import signal as sps
    mode = filter_mode(freqs)
    if mode == "all":
        return records
    f = [freqs] if isinstance(freqs, (int, float)) else list(freqs)
    wn = [2.0 * fr * dt for fr in f]
    b, a = sps.butter(order, wn[0] if len(wn) == 1 else wn, btype=mode)
    zi = sps.lfilter_zi(b, a)
    padlen = 3 * max(len(a), len(b))
    require_cuda(records, "filter_records")
    shape = records.shape
    x = records.reshape(shape[0], -1).contiguous().to(torch.float32)
    nt, ntr = x.shape
    if padlen >= nt:
        raise ValueError("records too short for the filter's padding")
    dev = records.device
    host = lambda v: torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).to(dev)
    bt, at, zt = host(b / a[0]), host(a / a[0]), host(zi)
    out = torch.empty_like(x)
    work = torch.empty(nt + 2 * padlen, ntr, dtype=torch.float64, device=dev)
    N.call("sgb_filtfilt", nt, ntr, len(b), N.ptr(bt), N.ptr(at), N.ptr(zt), padlen, N.ptr(x), N.ptr(out),
           N.ptr(work), N.stream_handle())
    return out.reshape(shape)
