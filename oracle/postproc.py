"""CPU oracle of the gradient post-processing and the L2 misfit.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restates
signal.gaussian_filter (signal.py:247-319) as applied by
PostProcess.smooth_gradient (process.py:66-113): a normalised Gaussian of
2r + 1 taps (r even) correlated along z then x over numpy 'reflect'
padding; PostProcess.precondition (process.py:115-118): grad / illum; and
loss.L2 (loss.py:409-421): sum over shots of sum (syn - obs)^2, gradient
2 (syn - obs).
"""
import numpy as np


def gaussian_taps(sigma, radius):
    ks = 2 * radius + 1 if radius % 2 == 0 else 2 * radius
    k = np.exp(-(np.arange(ks) - ks // 2) ** 2 / (2 * sigma ** 2))
    return k / k.sum()


def smooth_axis(a, sigma, radius, axis):
    k = gaussian_taps(sigma, radius)
    r = len(k) // 2
    pad = [(0, 0)] * a.ndim
    pad[axis] = (r, r)
    p = np.pad(np.asarray(a, np.float64), pad, mode="reflect")
    out = np.zeros(a.shape)
    n = a.shape[axis]
    for j in range(len(k)):
        sl = [slice(None)] * a.ndim
        sl[axis] = slice(j, j + n)
        out += k[j] * p[tuple(sl)]
    return out


def smooth_gradient(g, sigma, radius, counts):
    out = np.asarray(g, np.float64)
    for _ in range(counts):
        out = smooth_axis(out, sigma["z"], radius["z"], 0)
        out = smooth_axis(out, sigma["x"], radius["x"], 1)
    return out


def l2(syn, obs):
    d = np.asarray(syn, np.float64) - np.asarray(obs, np.float64)
    return float(np.sum(d * d)), 2.0 * d
