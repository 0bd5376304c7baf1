"""Golden vectors of the gradient post-processing and misfit, made by the
reference's own code: ``seistorch.signal.gaussian_filter`` applied the way
``PostProcess.smooth_gradient`` applies it (z then x, ``counts`` passes,
process.py:66-113), the illumination division of
``PostProcess.precondition`` (process.py:115-118) and ``loss.L2``
(loss.py:409-421).  Run here, where the reference tree exists; the fixture
is committed as postproc.npz."""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_loader as RL  # noqa: E402


def main():
    RL.load("cpu")
    import importlib
    sig = importlib.import_module("seistorch.signal")
    rng = np.random.default_rng(0)
    g = rng.standard_normal((40, 70)).astype(np.float32)
    illum = (rng.random((40, 70)) + 0.1).astype(np.float32)
    out = {"grad": g, "illum": illum}
    for name, sz, rz, sx, rx, counts in [("a", 2.0, 4, 3.0, 6, 1), ("b", 1.5, 2, 1.0, 2, 3)]:
        t = torch.tensor(g)
        for _ in range(counts):
            t = sig.gaussian_filter(t, sz, rz, axis=0)
            t = sig.gaussian_filter(t, sx, rx, axis=1)
        out["smooth_" + name] = t.numpy()
        out["smooth_" + name + "_par"] = np.array([sz, rz, sx, rx, counts], np.float64)
    out["precond"] = (torch.tensor(g) / torch.tensor(illum)).numpy()
    loss_mod = importlib.import_module("seistorch.loss")
    syn = [torch.tensor(rng.standard_normal((30, 5, 1)).astype(np.float32)) for _ in range(3)]
    obs = [torch.tensor(rng.standard_normal((30, 5, 1)).astype(np.float32)) for _ in range(3)]
    syn_g = [s.clone().requires_grad_(True) for s in syn]
    loss = loss_mod.L2()(syn_g, obs)
    loss.backward()
    out["l2_syn"] = np.stack([s.numpy() for s in syn])
    out["l2_obs"] = np.stack([o.numpy() for o in obs])
    out["l2_loss"] = np.array(loss.item())
    out["l2_grad"] = np.stack([s.grad.numpy() for s in syn_g])
    # non-linear conjugate gradient (optimizer.py:144-224): four steps of a
    # 40 x 70 parameter with a drawn gradient each, PR with the quantile
    # clamp and FR without it
    opt_mod = importlib.import_module("seistorch.optimizer")
    r2 = np.random.default_rng(1)
    p0 = (2000.0 + 100.0 * r2.standard_normal((40, 70))).astype(np.float32)
    grads = (r2.standard_normal((4, 40, 70)) * np.linspace(1.0, 3.0, 70)).astype(np.float32)
    out["ncg_p0"], out["ncg_grads"] = p0, grads
    for tag, beta, clamp in (("pr", "PR", True), ("fr", "FR", False)):
        prm = torch.nn.Parameter(torch.tensor(p0))
        opt = opt_mod.Cg([prm], lr=10.0, beta_type=beta, grad_clamp=clamp, clip_value=0.02)
        steps = []
        for k in range(4):
            prm.grad = torch.tensor(grads[k])
            opt.step()
            steps.append(prm.detach().numpy().copy())
        out["ncg_" + tag] = np.stack(steps)
    np.savez_compressed(os.path.join(HERE, "postproc.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
