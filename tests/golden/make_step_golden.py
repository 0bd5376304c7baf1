"""Golden vectors for the per-step drop-ins, made by running the reference's
own equation modules on CPU in float64.

Run in a container that holds the reference source tree::

    SEISTORCH_REF_ROOT=<reference checkout> python tests/golden/make_step_golden.py

For every case it stores seeded inputs (models, two time levels of smooth
random wavefields, a random output cotangent) and, from the reference:

* ``_time_step`` outputs and their autograd VJP (d<sum(y * gy)>/d(models,
  fields)) -- what autograd through ``WaveCell`` with
  ``boundary_saving: false`` computes each step (cell.py:74-75);
* ``_time_step_backward`` / ``_time_step_backward_multiple`` outputs with
  strips taken by ``save_boundaries`` and a source re-add, and their
  autograd VJP -- what ``CheckpointFunction.backward`` differentiates
  (checkpoint_new.py:180-199);
* ``save_boundaries`` / ``restore_boundaries`` results (equations2d/utils.py:50-90).

Outputs go to ``tests/golden/steps_<case>.npz``.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_loader as RL  # noqa: E402

W = 50  # the reference's HABC / strip-save width


def f32(a):
    """Inputs are rounded to float32 before the float64 reference runs, so
    the stored float32 copies are exactly the inputs it saw."""
    return np.asarray(a, np.float32).astype(np.float64)


def smooth_field(rng, shape, amp=1.0):
    from scipy.ndimage import gaussian_filter
    f = gaussian_filter(rng.standard_normal(shape), sigma=(0, 3, 3))
    return f32(amp * f / np.abs(f).max())


def layered(nz, nx, lo, hi, rng):
    m = np.linspace(lo, hi, nz)[:, None] * np.ones((1, nx))
    zz, xx = np.mgrid[0:nz, 0:nx]
    cz, cx = rng.uniform(0.3, 0.7) * nz, rng.uniform(0.3, 0.7) * nx
    return f32(m + 0.1 * (hi - lo) * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * (0.2 * min(nz, nx)) ** 2)))


CASES = {
    "acoustic_pml_o4": dict(equation="acoustic", order=4, habc=False, multiple=False),
    "acoustic_pml_o2_multiple": dict(equation="acoustic", order=2, habc=False, multiple=True),
    "acoustic_habc_o2": dict(equation="acoustic_habc", order=2, habc=True, multiple=False),
    "acoustic_habc_o4": dict(equation="acoustic_habc", order=4, habc=True, multiple=False),
    "acoustic_habc_o2_multiple": dict(equation="acoustic_habc", order=2, habc=True, multiple=True),
    "vti_habc2": dict(equation="vti_habc2", order=2, habc=True, multiple=False),
    "vti_habc2_multiple": dict(equation="vti_habc2", order=2, habc=True, multiple=True),
    "rho_habc": dict(equation="acoustic_rho_habc", order=2, habc=True, multiple=False),
    "born_habc_o2": dict(equation="acoustic_lsrtm_habc", order=2, habc=True, multiple=False),
    "born_habc_o4_multiple": dict(equation="acoustic_lsrtm_habc", order=4, habc=True, multiple=True),
    "elastic": dict(equation="elastic", order=2, habc=False, multiple=False),
    "vacoustic_habc": dict(equation="vacoustic_habc", order=2, habc=True, multiple=False),
    "vacoustic_habc_multiple": dict(equation="vacoustic_habc", order=2, habc=True, multiple=True),
}


def eq_module(ref, equation, order, dtype):
    mod = {"acoustic": ref.acoustic, "acoustic_habc": ref.acoustic_habc,
           "acoustic_lsrtm_habc": ref.acoustic_lsrtm_habc, "vti_habc2": ref.vti_habc2,
           "acoustic_rho_habc": ref.acoustic_rho_habc, "vacoustic_habc": ref.vacoustic_habc,
           "elastic": ref.elastic}[equation]
    if equation == "acoustic_rho_habc":
        for n in ("kernelx_gc_pos", "kernelx_gc_neg", "kernely_gc_pos", "kernely_gc_neg", "kernelx_gc_pos2",
                  "kernelx_gc_neg2", "kernely_gc_pos2", "kernely_gc_neg2"):
            setattr(mod, n, getattr(ref.convkernel, n).to(dtype))
    elif equation == "vti_habc2":
        mod.kernelx = ref.convkernel.kernelx.to(dtype)
        mod.kernely = ref.convkernel.kernely.to(dtype)
    elif equation == "acoustic_lsrtm_habc":
        RL.set_spatial_order(ref.acoustic_habc, order, dtype)
    elif equation != "elastic":
        RL.set_spatial_order(mod, order, dtype)
    return mod


def models_for(equation, nz, nx, rng):
    vp = layered(nz, nx, 1600.0, 3200.0, rng)
    if equation in ("acoustic", "acoustic_habc"):
        return {"vp": vp}
    if equation == "acoustic_lsrtm_habc":
        return {"vp": vp, "m": f32(0.05 * smooth_field(rng, (1, nz, nx))[0])}
    if equation == "vti_habc2":
        return {"vp": vp, "epsilon": f32(0.1 + 0.1 * layered(nz, nx, 0.0, 1.0, rng)),
                "delta": f32(0.05 + 0.05 * layered(nz, nx, 0.0, 1.0, rng))}
    if equation == "acoustic_rho_habc":
        return {"vp": vp, "rho": layered(nz, nx, 1000.0, 2400.0, rng)}
    if equation == "vacoustic_habc":
        return {"vp": vp, "Q": layered(nz, nx, 20.0, 80.0, rng)}
    vpe = layered(nz, nx, 2000.0, 3600.0, rng)
    return {"vp": vpe, "vs": f32(vpe / 1.73), "rho": f32(310.0 * vpe ** 0.25)}


def run(ref, name, equation, order, habc, multiple, B=2, nzi=8, nxi=12, seed=0):
    dtype = torch.float64
    torch.set_default_dtype(dtype)
    rng = np.random.default_rng(seed + 17 * list(CASES).index(name))
    mod = eq_module(ref, equation, order, dtype)
    top = 0 if multiple else W
    nz, nx = nzi + top + W, nxi + 2 * W
    models = models_for(equation, nz, nx, rng)
    names = ref.eqconfigure.Parameters.valid_model_paras()[equation]
    fields = ref.eqconfigure.Wavefield(equation).wavefields
    if equation == "elastic":
        dt, h = 0.0005, 5.0
    else:
        dt, h = 0.001, 10.0
    if habc:
        d = ref.habc.generate_habc_coefficients_2d((nz, nx), W, multiple=multiple)
        masks = ref.habc.bound_mask(nz, nx, W, "cpu", B, return_idx=True, multiple=multiple)
    else:
        d = ref.pml.generate_pml_coefficients_2d((nz, nx), W, multiple=multiple)
        masks = None
    d = torch.as_tensor(d, dtype=dtype)
    amp = {"vx": 1e-3, "vz": 1e-3}
    F = {f: smooth_field(rng, (B, nz, nx), amp.get(f, 1.0)) for f in fields}
    out = {"equation": np.array(equation), "order": np.array(order), "habc": np.array(habc),
           "multiple": np.array(multiple), "dt": np.array(dt), "h": np.array(h), "d": d.numpy(),
           "model_names": np.array(names), "field_names": np.array(fields)}
    for n in names:
        out["model_" + n] = models[n]
    for f in fields:
        out["in_" + f] = F[f]

    def tens(a):
        return torch.tensor(a, dtype=dtype, requires_grad=True)

    dtt = torch.tensor(dt, dtype=dtype)
    ht = torch.tensor(h, dtype=dtype)
    # outputs that are new time levels (second-order equations return (y, h1) pairs)
    second = equation != "elastic"
    outs_new = [0] if equation in ("acoustic", "acoustic_habc", "vti_habc2", "acoustic_rho_habc",
                                   "vacoustic_habc") else \
        ([0, 2] if equation == "acoustic_lsrtm_habc" else [0, 1, 2, 3, 4])
    G = [smooth_field(rng, (B, nz, nx), 1.0) for _ in outs_new]
    for i, g in zip(outs_new, G):
        out[f"gy_{i}"] = g

    # --- forward step and its VJP
    mt = [tens(models[n]) for n in names]
    ft = [tens(F[f]) for f in fields]
    y = mod._time_step(*mt, *ft, dtt, ht, d, habcs=masks)
    loss = sum((y[i] * torch.as_tensor(g)).sum() for i, g in zip(outs_new, G))
    loss.backward()
    for i in outs_new:
        out[f"step_out_{i}"] = y[i].detach().numpy()
    for n, t in zip(names, mt):
        out["step_grad_" + n] = t.grad.numpy()
    for f, t in zip(fields, ft):
        out["step_grad_" + f] = t.grad.numpy()

    # --- reverse step (boundary-saving path): strips of a random state, a source re-add
    nxt = {f: smooth_field(rng, (B, nz, nx), amp.get(f, 1.0)) for f in fields}
    strips = [RL_save(ref, torch.as_tensor(nxt[f])) for f in fields]
    for f, st in zip(fields, strips):
        for k, s in zip("tblr", st):
            out[f"strip_{f}_{k}"] = s.numpy()
    smask = np.zeros((B, nz, nx))
    for b in range(B):
        smask[b, top + 2, W + 3 + 7 * b] = 1.0
    sval = np.array([[0.37]])  # one wavelet sample shared by the shots, as rnn.py:186 passes it
    out["smask"] = smask
    out["src_value"] = sval
    sm = torch.as_tensor(smask)
    sv = torch.as_tensor(sval)

    def src_func(Y, X, dt_=1.0):
        return Y + sm * X

    src_type = ["vx"] if equation == "elastic" else [fields[0]]
    out["src_type"] = np.array(src_type)
    mt = [tens(models[n]) for n in names]
    ft = [tens(F[f]) for f in fields]
    back = mod._time_step_backward_multiple if multiple and equation != "elastic" else mod._time_step_backward
    yb = back(*mt, *ft, dtt, ht, d, strips, [src_type, src_func, sv])
    rev_new = outs_new
    for i in rev_new:
        out[f"rev_out_{i}"] = yb[i].detach().numpy()
    if equation != "elastic":
        lossb = sum((yb[i] * torch.as_tensor(g)).sum() for i, g in zip(rev_new, G))
        lossb.backward()
        for n, t in zip(names, mt):
            out["rev_grad_" + n] = t.grad.numpy() if t.grad is not None else np.zeros_like(models[n])
        for f, t in zip(fields, ft):
            out["rev_grad_" + f] = t.grad.numpy() if t.grad is not None else np.zeros_like(F[f])

    # --- strip utilities on their own
    u = torch.as_tensor(F[fields[0]]).clone()
    s = ref.utils2d.save_boundaries(u)
    tgt = torch.as_tensor(nxt[fields[0]]).clone()
    out["restored"] = ref.utils2d.restore_boundaries(tgt.clone(), s).numpy()
    out["restored_multiple"] = ref.utils2d.restore_boundaries(tgt.clone(), s, multiple=True).numpy()
    out["restore_target"] = tgt.numpy()
    torch.set_default_dtype(torch.float32)
    return out


def RL_save(ref, t):
    return tuple(s.clone() for s in ref.utils2d.save_boundaries(t))


def main(only=None):
    ref = RL.load("cpu")
    for name, kw in CASES.items():
        if only and name not in only:
            continue
        res = run(ref, name, **kw)
        # float32 storage: the inputs are float32 values, the float64 outputs
        # keep 7 digits, far inside the 1e-5 tolerances of the tests
        res = {k: (v.astype(np.float32) if v.dtype == np.float64 and v.ndim > 0 else v) for k, v in res.items()}
        np.savez_compressed(os.path.join(HERE, f"steps_{name}.npz"), **res)
        print(name, sorted(k for k in res if k.startswith(("step_grad", "rev_grad", "rev_out", "step_out"))))


if __name__ == "__main__":
    main(sys.argv[1:] or None)
