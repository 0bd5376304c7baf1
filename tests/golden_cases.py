"""Helpers that turn a golden ``.npz`` (made by tests/golden/make_golden.py
from the reference's own code) back into inputs for the oracle and the GPU
path."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

FORWARD_CASES = ["acoustic_pml_o2", "acoustic_pml_o4", "acoustic_pml_o8",
                 "acoustic_pml_o4_multiple", "acoustic_habc_o2", "acoustic_habc_o4",
                 "acoustic_habc_o2_multiple", "elastic", "elastic_multiple",
                 "born_habc_o2", "born_habc_o4", "born_habc_o2_multiple", "vti_habc2", "vti_habc2_multiple",
                 "rho_habc", "rho_habc_multiple", "vacoustic_habc", "vacoustic_habc_multiple"]
GRAD_CASES = ["grad_acoustic_pml_o4", "grad_acoustic_pml_o8", "grad_elastic"]
BORN_GRAD_CASES = ["grad_born_habc_o2_zeroobs", "grad_born_habc_o4"]
VTI_GRAD_CASES = ["grad_vti_habc2_zeroobs"]
RHO_GRAD_CASES = ["grad_rho_habc_zeroobs"]
MODEL_PARAMS = {"acoustic": ["vp"], "acoustic_habc": ["vp"], "acoustic_lsrtm_habc": ["vp", "m"],
                "vti_habc2": ["vp", "epsilon", "delta"], "acoustic_rho_habc": ["vp", "rho"],
                "vacoustic_habc": ["vp", "Q"],
                "elastic": ["vp", "vs", "rho"]}


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["equation"] = str(g["equation"])
    for k in ("order", "width", "nt", "nshots"):
        g[k] = int(g[k])
    for k in ("dt", "h", "fm"):
        g[k] = float(g[k])
    for k in ("multiple", "habc"):
        g[k] = bool(g[k])
    g["source_type"] = [str(s) for s in g["source_type"]]
    g["receiver_type"] = [str(s) for s in g["receiver_type"]]
    g["models"] = {n: g["model_" + n] for n in MODEL_PARAMS[g["equation"]]}
    g["sources"] = [[(int(z_), int(x_))] for z_, x_ in g["src"]]
    g["receivers"] = [(list(map(int, zs)), list(map(int, xs)))
                      for zs, xs in zip(g["rec_z"], g["rec_x"])]
    return g


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
