"""CPU oracle of the learned preconditioner network (seistorch_gb300.learned).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  The network has no
counterpart in the reference; this restates the same 4-level network in
numpy float64 -- forward and exact backward -- with the activations and
gradients rounded to bfloat16 at the points where the GPU stores them, so
the GPU kernels can be checked layer for layer.  Parameters use the same
flat layout: per layer W [cout][cin][3][3] then b [cout].
"""
import numpy as np

LAYERS = [("e1a", 2, 32), ("e1b", 32, 32), ("e2a", 32, 64), ("e2b", 64, 64), ("e3a", 64, 128),
          ("e3b", 128, 128), ("b4", 128, 256), ("d3", 384, 128), ("d2", 192, 64), ("d1", 96, 32), ("out", 32, 1)]
TENSOR_CORE = {"e1b", "e2a", "e2b", "e3a", "e3b", "b4", "d3", "d2", "d1"}


def _round(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, off = {}, 0
    for name, ci, co in LAYERS:
        n = ci * co * 9
        out[name] = (params[off:off + n].reshape(co, ci, 3, 3).astype(np.float64),
                     params[off + n:off + n + co].astype(np.float64))
        off += n + co
    return out


def _shift(x, dy, dx):
    """x[..., y + dy, x + dx] with zeros outside (x: [..., H, W])."""
    out = np.zeros_like(x)
    H, W = x.shape[-2:]
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[..., yd, xd] = x[..., ys, xs]
    return out


def conv(x, W, b=None):
    """3x3 convolution, zero padding 1; x [B][C][H][W], W [O][C][3][3]."""
    y = np.zeros((x.shape[0], W.shape[0]) + x.shape[2:])
    for ky in range(3):
        for kx in range(3):
            y += np.einsum("oc,bchw->bohw", W[:, :, ky, kx], _shift(x, ky - 1, kx - 1))
    if b is not None:
        y += b[None, :, None, None]
    return y


def conv_bwd(x, W, g):
    """(dx, dW, db) of y = conv(x, W) + b for dL/dy = g."""
    dx = np.zeros_like(x)
    dW = np.zeros_like(W)
    for ky in range(3):
        for kx in range(3):
            xs = _shift(x, ky - 1, kx - 1)
            dW[:, :, ky, kx] = np.einsum("bohw,bchw->oc", g, xs)
            dx += _shift(np.einsum("oc,bohw->bchw", W[:, :, ky, kx], g), 1 - ky, 1 - kx)
    return dx, dW, g.sum(axis=(0, 2, 3))


def pool(x):
    B, C, H, W = x.shape
    return x.reshape(B, C, H // 2, 2, W // 2, 2).mean(axis=(3, 5))


def up(x):
    return x.repeat(2, axis=2).repeat(2, axis=3)


def forward(params, x, rounding=True):
    """x [B][2][H][W] -> (prediction [B][H][W], cache).  rounding=False
    keeps everything in float64 (exact network, for finite differences)."""
    bf16 = _round if rounding else (lambda a: np.asarray(a, np.float64))
    P = unpack(params)
    Wb = {k: (bf16(w) if k in TENSOR_CORE else w, b) for k, (w, b) in P.items()}
    relu = lambda a: np.maximum(a, 0.0)
    c = {"x": x}
    c["a1a"] = bf16(relu(conv(x, *Wb["e1a"])))
    c["s1"] = bf16(relu(conv(c["a1a"], *Wb["e1b"])))
    c["p1"] = bf16(pool(c["s1"]))
    c["a2a"] = bf16(relu(conv(c["p1"], *Wb["e2a"])))
    c["s2"] = bf16(relu(conv(c["a2a"], *Wb["e2b"])))
    c["p2"] = bf16(pool(c["s2"]))
    c["a3a"] = bf16(relu(conv(c["p2"], *Wb["e3a"])))
    c["s3"] = bf16(relu(conv(c["a3a"], *Wb["e3b"])))
    c["p3"] = bf16(pool(c["s3"]))
    c["a4"] = bf16(relu(conv(c["p3"], *Wb["b4"])))
    c["cat3"] = np.concatenate([up(c["a4"]), c["s3"]], axis=1)
    c["ad3"] = bf16(relu(conv(c["cat3"], *Wb["d3"])))
    c["cat2"] = np.concatenate([up(c["ad3"]), c["s2"]], axis=1)
    c["ad2"] = bf16(relu(conv(c["cat2"], *Wb["d2"])))
    c["cat1"] = np.concatenate([up(c["ad2"]), c["s1"]], axis=1)
    c["ad1"] = bf16(relu(conv(c["cat1"], *Wb["d1"])))
    pred = conv(c["ad1"], *Wb["out"])[:, 0]
    c["Wb"] = Wb
    c["round"] = bf16
    return pred, c


def backward(params, cache, dpred):
    """Flat gradient of sum(pred * dpred)."""
    Wb = cache["Wb"]
    bf16 = cache["round"]
    grads = {}
    mask = lambda g, a: np.where(a > 0, g, 0.0)
    upb = lambda g: g.reshape(g.shape[0], g.shape[1], g.shape[2] // 2, 2, g.shape[3] // 2, 2).sum(axis=(3, 5))

    def layer(name, x, g):
        dx, dW, db = conv_bwd(x, Wb[name][0], g)
        grads[name] = (dW, db)
        return dx

    g = dpred[:, None]
    d = layer("out", cache["ad1"], g)
    g1 = bf16(mask(d, cache["ad1"]))
    dcat1 = layer("d1", cache["cat1"], g1)
    g2 = bf16(mask(upb(dcat1[:, :64]), cache["ad2"]))
    dcat2 = layer("d2", cache["cat2"], g2)
    g3 = bf16(mask(upb(dcat2[:, :128]), cache["ad3"]))
    dcat3 = layer("d3", cache["cat3"], g3)
    g4 = bf16(mask(upb(dcat3[:, :256]), cache["a4"]))
    dp3 = layer("b4", cache["p3"], g4)
    g3b = bf16(mask(0.25 * up(dp3) + dcat3[:, 256:], cache["s3"]))
    d = layer("e3b", cache["a3a"], g3b)
    g3a = bf16(mask(d, cache["a3a"]))
    dp2 = layer("e3a", cache["p2"], g3a)
    g2b = bf16(mask(0.25 * up(dp2) + dcat2[:, 128:], cache["s2"]))
    d = layer("e2b", cache["a2a"], g2b)
    g2a = bf16(mask(d, cache["a2a"]))
    dp1 = layer("e2a", cache["p1"], g2a)
    g1b = bf16(mask(0.25 * up(dp1) + dcat1[:, 64:], cache["s1"]))
    d = layer("e1b", cache["a1a"], g1b)
    g1a = bf16(mask(d, cache["a1a"]))
    layer("e1a", cache["x"], g1a)
    out = []
    for name, ci, co in LAYERS:
        dW, db = grads[name]
        out += [dW.reshape(-1), db.reshape(-1)]
    return np.concatenate(out)
