"""Pin the oracle's discrete adjoints against the reference's autograd
gradients (golden vectors) and against finite differences."""
import numpy as np
import pytest

from oracle import adjoint, fd2d
from tests.golden_cases import load, rel_l2


def _l2_record_grads(g, models):
    out = fd2d.forward(g["equation"], models, g["d"], g["dt"], g["h"], g["wavelet"],
                       g["sources"], g["receivers"], order=g["order"])
    syn = np.stack(out["records"])
    return syn, [2.0 * (s - o) for s, o in zip(syn, g["obs"])]


@pytest.mark.parametrize("name", ["grad_acoustic_pml_o4", "grad_acoustic_pml_o8"])
def test_acoustic_adjoint_matches_reference_autograd(name):
    g = load(name)
    syn, rg = _l2_record_grads(g, g["models"])
    assert rel_l2(syn, g["records"]) < 1e-11
    loss = float(np.sum((syn - g["obs"]) ** 2))
    assert abs(loss - float(g["loss"])) < 1e-9 * abs(float(g["loss"]))
    grad = adjoint.acoustic_pml_gradient(g["models"]["vp"], g["d"], g["dt"], g["h"], g["wavelet"],
                                         g["sources"], g["receivers"], rg, order=g["order"])
    assert rel_l2(grad, g["grad_vp"]) < 1e-10


def test_elastic_adjoint_matches_reference_autograd():
    g = load("grad_elastic")
    syn, rg = _l2_record_grads(g, g["models"])
    assert rel_l2(syn, g["records"]) < 1e-11
    gvp, gvs, grho = adjoint.elastic_gradient(g["models"]["vp"], g["models"]["vs"],
                                              g["models"]["rho"], g["d"], g["dt"], g["h"],
                                              g["wavelet"], g["sources"], g["receivers"], rg)
    assert rel_l2(gvp, g["grad_vp"]) < 1e-9
    assert rel_l2(gvs, g["grad_vs"]) < 1e-9
    assert rel_l2(grho, g["grad_rho"]) < 1e-9


def test_acoustic_adjoint_matches_finite_difference():
    g = load("grad_acoustic_pml_o4")
    vp = g["models"]["vp"]
    _, rg = _l2_record_grads(g, g["models"])
    grad = adjoint.acoustic_pml_gradient(vp, g["d"], g["dt"], g["h"], g["wavelet"], g["sources"],
                                         g["receivers"], rg, order=4)

    def loss(v):
        syn, _ = _l2_record_grads(g, {"vp": v})
        return float(np.sum((syn - g["obs"]) ** 2))
    for (z, x) in [(25, 30), (35, 50), (22, 40)]:
        eps = 1e-3
        vpp = vp.copy()
        vpp[z, x] += eps
        vpm = vp.copy()
        vpm[z, x] -= eps
        fd = (loss(vpp) - loss(vpm)) / (2 * eps)
        assert abs(fd - grad[z, x]) <= 1e-6 * abs(grad).max()


def test_checkpointed_oracle_adjoint_is_identical():
    """keep_every recomputes the forward segments in the reverse sweep with
    the same float64 arithmetic: the gradient is bit-identical to keeping
    every state (segment lengths that divide nt, do not, and exceed it)."""
    import numpy as np
    from oracle import adjoint, fd2d
    rng = np.random.default_rng(3)
    nz, nx, w = 36, 44, 10
    vp = 1800 + 400 * rng.random((nz, nx))
    d = fd2d.pml_profile_2d((nz, nx), w)
    wav = fd2d.ricker(15, 0.001, 90, delay=30)
    src = [[(w + 2, w + 5)], [(w + 2, w + 18)]]
    rec = [([w + 1] * 8, list(range(w, w + 24, 3)))] * 2
    rg = [rng.standard_normal((90, 8, 1)) for _ in range(2)]
    full = adjoint.acoustic_pml_gradient(vp, d, 0.001, 10, wav, src, rec, rg, order=8)
    for S in (1, 9, 13, 200):
        part = adjoint.acoustic_pml_gradient(vp, d, 0.001, 10, wav, src, rec, rg, order=8, keep_every=S)
        assert np.array_equal(full, part), S
