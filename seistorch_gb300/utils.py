"""Small helpers with seistorch's names (seistorch/utils.py)."""
import numpy as np
import torch


def ricker_wave(fm, dt, T, delay=80, dtype="tensor", inverse=False):
    """Ricker wavelet p(1-2c^2)exp(-c^2), c = pi fm (i dt - delay dt), rounded
    to float32 (utils.py:235-249)."""
    i = np.arange(T, dtype=np.float64)
    c = np.pi * fm * (i * dt - delay * dt)
    p = -1.0 if inverse else 1.0
    w = (p * (1 - 2 * c ** 2) * np.exp(-c ** 2)).astype(np.float32)
    return w if dtype == "numpy" else torch.from_numpy(w)


def set_dtype(dtype=None):
    if dtype == "float32" or dtype is None:
        torch.set_default_dtype(torch.float32)
    elif dtype == "float64":
        torch.set_default_dtype(torch.float64)
    else:
        raise ValueError(f"Unsupported data type: {dtype}; should be either float32 or float64")


def to_tensor(x, dtype=None):
    dtype = dtype if dtype is not None else torch.get_default_dtype()
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().to(dtype)
    if isinstance(x, (float, int)):
        return torch.tensor(x).type(dtype)
    if isinstance(x, list):
        if None in x:
            return torch.Tensor([])
        x = np.array([i.cpu().numpy() if hasattr(i, "device") else i for i in x])
    return torch.from_numpy(np.asarray(x)).type(dtype)


def update_cfg(cfg, geom="geom", device="cpu"):
    """Grow Nx/Ny by the boundary width (top unpadded with ``multiple``) and
    set ``domain_shape`` (utils.py:282-329, 2D)."""
    vel = cfg.get("VEL_PATH") or {}
    for path in vel.values():
        if path is None:
            continue
        d = np.load(path) if isinstance(path, str) else np.asarray(path)
        ny, nx = d.shape[-2:]
        cfg[geom].update({"Nx": nx, "Ny": ny, "Nz": 0})
        break
    Nx, Ny = cfg[geom]["Nx"], cfg[geom]["Ny"]
    pad = cfg[geom]["boundary"]["width"]
    multiple = cfg[geom].get("multiple", False)
    cfg[geom]["_oriNx"], cfg[geom]["_oriNy"], cfg[geom]["_oriNz"] = Nx, Ny, 0
    cfg[geom]["Nx"] = Nx + 2 * pad
    cfg[geom]["Ny"] = Ny + pad if multiple else Ny + 2 * pad
    cfg["domain_shape"] = (cfg[geom]["Ny"], cfg[geom]["Nx"])
    cfg["device"] = device
    return cfg
