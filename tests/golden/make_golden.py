"""Generate golden vectors by running the reference seistorch code on CPU.

Run in a container that holds the reference source tree (see
``ref_loader.REF_ROOT``)::

    SEISTORCH_REF_ROOT=<reference checkout> python tests/golden/make_golden.py

Each case runs the reference ``WaveRNN``/``WaveCell`` time loop
(rnn.py:100-217, cell.py:50-77) with its own equation modules, PML/HABC
coefficient generators and sources/probes, in float64 and float32, and saves
records, final wavefields and (for the gradient cases) the reference's pure
autograd gradient (``boundary_saving: false``) of an L2 misfit
(loss.py:409-421, ``MSELoss(reduction='sum')``).  Outputs go to
``tests/golden/*.npz``; the inputs needed to re-run a case are stored in the
same file, so the tests never need the reference.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_loader as RL  # noqa: E402


def layered(nz, nx, vals, seed, anomaly=150.0):
    rng = np.random.default_rng(seed)
    m = np.zeros((nz, nx))
    bounds = np.linspace(0, nz, len(vals) + 1).astype(int)
    for v, a, b in zip(vals, bounds[:-1], bounds[1:]):
        m[a:b] = v
    zz, xx = np.mgrid[0:nz, 0:nx]
    cz, cx = rng.uniform(0.3, 0.7) * nz, rng.uniform(0.3, 0.7) * nx
    m += anomaly * np.exp(-((zz - cz) ** 2 + (xx - cx) ** 2) / (2 * (0.15 * min(nz, nx)) ** 2))
    return m


def acquisition(nz_int, nx_int, nshots, width, multiple, step=3):
    top = 0 if multiple else width
    src = []
    rec = []
    for s in range(nshots):
        x = width + 2 + s * max(1, (nx_int - 4) // max(1, nshots))
        src.append((top + 2, x))
        xs = list(range(width, width + nx_int, step))
        rec.append(([top + 1] * len(xs), xs))
    return src, rec


def run_case(ref, equation, models_int, *, order=2, width=20, multiple=False, nshots=2,
             nt=200, dt=0.001, h=10.0, fm=15.0, habc=False, dtype=torch.float64,
             grad=None, obs_models=None, source_type=None, receiver_type=None, boundary_saving=False):
    torch.set_default_dtype(dtype)
    eqmod = {"acoustic": ref.acoustic, "acoustic_habc": ref.acoustic_habc,
             "acoustic_lsrtm_habc": ref.acoustic_lsrtm_habc, "vti_habc2": ref.vti_habc2,
             "acoustic_rho_habc": ref.acoustic_rho_habc, "vacoustic_habc": ref.vacoustic_habc,
             "elastic": ref.elastic}[equation]
    if equation == "acoustic_rho_habc":
        # its one-cell difference / averaging kernels (convkernel.py:79-89) in the run's dtype
        for n in ("kernelx_gc_pos", "kernelx_gc_neg", "kernely_gc_pos", "kernely_gc_neg", "kernelx_gc_pos2",
                  "kernelx_gc_neg2", "kernely_gc_pos2", "kernely_gc_neg2"):
            setattr(eqmod, n, getattr(ref.convkernel, n).to(dtype))
    elif equation == "vti_habc2":
        # its 1-D kernels (convkernel.py:73-74, fixed 2nd order) in the run's dtype
        eqmod.kernelx = ref.convkernel.kernelx.to(dtype)
        eqmod.kernely = ref.convkernel.kernely.to(dtype)
    elif equation == "acoustic_lsrtm_habc":
        # its Laplacian is acoustic_habc._laplacian, which reads acoustic_habc's kernel
        RL.set_spatial_order(ref.acoustic_habc, order, dtype)
    elif equation != "elastic":
        RL.set_spatial_order(eqmod, order, dtype)
    names = ref.eqconfigure.Parameters.valid_model_paras()[equation]
    top = 0 if multiple else width
    padded = {n: np.pad(models_int[n], ((top, width), (width, width)), mode="edge") for n in names}
    nz, nx = padded[names[0]].shape
    if habc:
        d = ref.habc.generate_habc_coefficients_2d((nz, nx), width, multiple=multiple)
    else:
        d = ref.pml.generate_pml_coefficients_2d((nz, nx), width, multiple=multiple)
    nz_i, nx_i = models_int[names[0]].shape
    src, rec = acquisition(nz_i, nx_i, nshots, width, multiple)
    w = ref.rutils.ricker_wave(fm, dt, nt, delay=int(1.2 / fm / dt), dtype="numpy")
    st = source_type or (["h1"] if equation != "elastic" else ["txx", "tzz"])
    rt = receiver_type or (["h1"] if equation != "elastic" else ["vx", "vz"])

    # model.py:87 marks the second-order equations' step function; the
    # boundary-saving reverse sweep reads it (checkpoint_new.py:147)
    eqmod._time_step.ACOUSTIC2nd = equation in ref.eqconfigure.Parameters.secondorder_equations()

    def forward(models, requires_grad=()):
        geom = RL.make_geom(ref, equation, models, d, dt, h, use_habc=habc, bwidth=width,
                            multiple=multiple, source_type=st, receiver_type=rt,
                            inversion=bool(requires_grad), requires_grad=requires_grad,
                            boundary_saving=boundary_saving and bool(requires_grad), dtype=dtype)
        # the reverse sweep's class-level state (checkpoint_new.py:111-112,
        # checkpoint.py:110-111) starts fresh for every case
        for ck in (ref.checkpoint_new.CheckpointFunction, ref.checkpoint.CheckpointFunction):
            ck.counts = 0
            ck.wavefields = []
        rnn, y = RL.run_wavernn(ref, geom, eqmod._time_step, eqmod._time_step_backward, w, src, rec)
        return geom, rnn, y

    out = {}
    if grad is None:
        with torch.no_grad():
            _, rnn, y = forward(padded)
        out["records"] = np.stack([t.numpy() for t in y.data])
        names_wf = ref.eqconfigure.Wavefield(equation).wavefields
        for n in names_wf:
            out["field_" + n] = getattr(rnn, n).numpy()[0]  # shot 0 keeps fixtures small
    else:
        if obs_models is None:
            # zero observed data: J = sum(syn^2), a residual free of cancellation
            obs_padded = padded
            with torch.no_grad():
                _, _, yobs = forward(obs_padded)
            obs = [torch.zeros_like(t) for t in yobs.data]
        else:
            obs_padded = {n: np.pad(obs_models[n], ((top, width), (width, width)), mode="edge")
                          for n in names}
            with torch.no_grad():
                _, _, yobs = forward(obs_padded)
            obs = [t.clone() for t in yobs.data]
        geom, rnn, y = forward(padded, requires_grad=tuple(grad))
        loss = sum(torch.nn.functional.mse_loss(s, o, reduction="sum") for s, o in zip(y.data, obs))
        loss.backward()
        out["records"] = np.stack([t.detach().numpy() for t in y.data])
        out["obs"] = np.stack([t.numpy() for t in obs])
        out["loss"] = np.array(loss.item())
        for n in grad:
            out["grad_" + n] = getattr(geom, n).grad.numpy()
        for n in names:
            out["obsmodel_" + n] = obs_padded[n]
    meta = dict(equation=equation, order=order, width=width, multiple=multiple, nt=nt, dt=dt,
                boundary_saving=boundary_saving,
                h=h, fm=fm, habc=habc, src=np.array(src), nshots=nshots,
                rec_z=np.array([r[0] for r in rec]), rec_x=np.array([r[1] for r in rec]),
                wavelet=w, d=np.asarray(d.numpy() if torch.is_tensor(d) else d),
                source_type=np.array(st), receiver_type=np.array(rt))
    for n in names:
        meta["model_" + n] = padded[n]
    out.update({k: np.asarray(v) for k, v in meta.items()})
    return out


def cases():
    a = {"vp": layered(20, 36, [1500.0, 2200.0, 3000.0], 0)}
    ah = {"vp": layered(16, 24, [1500.0, 2500.0], 1)}
    vp_e = layered(20, 36, [2000.0, 2800.0, 3600.0], 2)
    e = {"vp": vp_e, "vs": vp_e / 1.73, "rho": 310.0 * vp_e ** 0.25}
    a_obs = {"vp": layered(20, 36, [1500.0, 2200.0, 3000.0], 0, anomaly=0.0)}
    vp_eo = layered(20, 36, [2000.0, 2800.0, 3600.0], 2, anomaly=0.0)
    e_obs = {"vp": vp_eo, "vs": vp_eo / 1.73, "rho": 310.0 * vp_eo ** 0.25}
    C = {}
    for order in (2, 4, 8):
        C[f"acoustic_pml_o{order}"] = dict(equation="acoustic", models_int=a, order=order)
    C["acoustic_pml_o4_multiple"] = dict(equation="acoustic", models_int=a, order=4, multiple=True)
    C["acoustic_habc_o2"] = dict(equation="acoustic_habc", models_int=ah, order=2, width=50,
                                 habc=True, nt=240)
    C["acoustic_habc_o4"] = dict(equation="acoustic_habc", models_int=ah, order=4, width=50,
                                 habc=True, nt=240)
    C["acoustic_habc_o2_multiple"] = dict(equation="acoustic_habc", models_int=ah, order=2,
                                          width=50, habc=True, multiple=True, nt=240)
    C["elastic"] = dict(equation="elastic", models_int=e, dt=0.0005, h=5.0, fm=20.0, nt=300)
    C["elastic_multiple"] = dict(equation="elastic", models_int=e, dt=0.0005, h=5.0, fm=20.0,
                                 nt=300, multiple=True)
    C["grad_acoustic_pml_o4"] = dict(equation="acoustic", models_int=a, order=4, nt=150,
                                     grad=["vp"], obs_models=a_obs)
    C["grad_acoustic_pml_o8"] = dict(equation="acoustic", models_int=a, order=8, nt=150,
                                     grad=["vp"], obs_models=a_obs)
    C["grad_acoustic_pml_o4_zeroobs"] = dict(equation="acoustic", models_int=a, order=4, nt=150,
                                             grad=["vp"], obs_models=None)
    C["grad_acoustic_pml_o8_zeroobs"] = dict(equation="acoustic", models_int=a, order=8, nt=150,
                                             grad=["vp"], obs_models=None)
    C["grad_acoustic_habc_o2_zeroobs"] = dict(equation="acoustic_habc", models_int=ah, order=2, width=50,
                                              habc=True, nt=200, grad=["vp"], obs_models=None)
    C["grad_acoustic_habc_o4_zeroobs"] = dict(equation="acoustic_habc", models_int=ah, order=4, width=50,
                                              habc=True, nt=200, grad=["vp"], obs_models=None)
    C["grad_acoustic_habc_o2_multiple_zeroobs"] = dict(equation="acoustic_habc", models_int=ah, order=2,
                                                       width=50, habc=True, multiple=True, nt=200, grad=["vp"],
                                                       obs_models=None)
    born = {"vp": ah["vp"], "m": layered(16, 24, [0.0, 0.08, -0.05], 3, anomaly=0.04)}
    born_obs = {"vp": ah["vp"], "m": layered(16, 24, [0.0, 0.06, -0.02], 4, anomaly=0.0)}
    for order in (2, 4):
        C[f"born_habc_o{order}"] = dict(equation="acoustic_lsrtm_habc", models_int=born, order=order, width=50,
                                        habc=True, nt=240, receiver_type=["sh1"])
    C["born_habc_o2_multiple"] = dict(equation="acoustic_lsrtm_habc", models_int=born, order=2, width=50,
                                      habc=True, multiple=True, nt=240, receiver_type=["sh1"])
    C["grad_born_habc_o2_zeroobs"] = dict(equation="acoustic_lsrtm_habc", models_int=born, order=2, width=50,
                                          habc=True, nt=200, grad=["m"], obs_models=None, receiver_type=["sh1"])
    C["grad_born_habc_o4"] = dict(equation="acoustic_lsrtm_habc", models_int=born, order=4, width=50,
                                  habc=True, nt=200, grad=["m"], obs_models=born_obs, receiver_type=["sh1"])
    vti = {"vp": ah["vp"], "epsilon": layered(16, 24, [0.1, 0.2], 5, anomaly=0.05),
           "delta": layered(16, 24, [0.05, 0.1], 6, anomaly=0.02)}
    C["vti_habc2"] = dict(equation="vti_habc2", models_int=vti, order=2, width=50, habc=True, nt=240,
                          source_type=["p1"], receiver_type=["p1"])
    C["vti_habc2_multiple"] = dict(equation="vti_habc2", models_int=vti, order=2, width=50, habc=True,
                                   multiple=True, nt=240, source_type=["p1"], receiver_type=["p1"])
    C["grad_vti_habc2_zeroobs"] = dict(equation="vti_habc2", models_int=vti, order=2, width=50, habc=True, nt=200,
                                       grad=["vp", "epsilon", "delta"], obs_models=None, source_type=["p1"],
                                       receiver_type=["p1"])
    rho = {"vp": ah["vp"], "rho": layered(16, 24, [1000.0, 2200.0], 7, anomaly=300.0)}
    C["rho_habc"] = dict(equation="acoustic_rho_habc", models_int=rho, order=2, width=50, habc=True, nt=240)
    C["rho_habc_multiple"] = dict(equation="acoustic_rho_habc", models_int=rho, order=2, width=50, habc=True,
                                  multiple=True, nt=240)
    C["grad_rho_habc_zeroobs"] = dict(equation="acoustic_rho_habc", models_int=rho, order=2, width=50, habc=True,
                                      nt=200, grad=["vp", "rho"], obs_models=None)
    # the reference's per-step boundary-saving gradient (cell.py:71-72; 1-cell
    # strips at index 49, so a 50-cell boundary)
    C["grad_bs_acoustic_pml_o2_zeroobs"] = dict(equation="acoustic", models_int=ah, order=2, width=50, nt=160,
                                                grad=["vp"], obs_models=None, boundary_saving=True)
    C["grad_bs_acoustic_habc_o2_zeroobs"] = dict(equation="acoustic_habc", models_int=ah, order=2, width=50,
                                                 habc=True, nt=160, grad=["vp"], obs_models=None,
                                                 boundary_saving=True)
    C["grad_bs_elastic_zeroobs"] = dict(equation="elastic", models_int=e, dt=0.0005, h=5.0, fm=20.0, width=50,
                                        nt=160, grad=["vp", "vs", "rho"], obs_models=None, boundary_saving=True)
    vac = {"vp": ah["vp"], "Q": layered(16, 24, [25.0, 60.0], 8, anomaly=10.0)}
    C["vacoustic_habc"] = dict(equation="vacoustic_habc", models_int=vac, order=2, width=50, habc=True, nt=240)
    C["vacoustic_habc_multiple"] = dict(equation="vacoustic_habc", models_int=vac, order=2, width=50, habc=True,
                                        multiple=True, nt=240)
    C["grad_vacoustic_habc_zeroobs"] = dict(equation="vacoustic_habc", models_int=vac, order=2, width=50,
                                            habc=True, nt=160, grad=["vp", "Q"], obs_models=None)
    C["grad_elastic_zeroobs"] = dict(equation="elastic", models_int=e, dt=0.0005, h=5.0, fm=20.0,
                                     nt=200, grad=["vp", "vs", "rho"], obs_models=None)
    C["grad_elastic"] = dict(equation="elastic", models_int=e, dt=0.0005, h=5.0, fm=20.0,
                             nt=200, grad=["vp", "vs", "rho"], obs_models=e_obs)
    return C


def main(only=None):
    ref = RL.load("cpu")
    for name, kw in cases().items():
        if only and name not in only:
            continue
        res64 = run_case(ref, dtype=torch.float64, **kw)
        if kw.get("grad") is None:
            res32 = run_case(ref, dtype=torch.float32, **kw)
            res64["records_f32"] = res32["records"]
            for k in list(res32):
                if k.startswith("field_"):
                    res64[k + "_f32"] = res32[k]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res64)
        print(name, {k: v.shape for k, v in res64.items() if k.startswith(("records", "grad"))})
    torch.set_default_dtype(torch.float32)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
