"""Pin the gradient goldens of the neighbouring equations (Born modelling,
VTI, variable density) independently of the reference's autograd: central
finite differences of the fp64 oracle's misfit J = sum(records^2) (the
goldens' zero-observation case, full length: 200 steps, 116 x 124, two
shots) at the two cells of largest gradient inside the undamped box agree
with the golden gradient to 1e-4 relative.  The oracle's forward matches
the reference's records to 1e-11, so this checks the goldens' adjoint."""
import numpy as np
import pytest

from oracle import fd2d
from tests.golden_cases import load

CASES = [("grad_born_habc_o2_zeroobs", "m", 1e-4), ("grad_vti_habc2_zeroobs", "epsilon", 1e-5),
         ("grad_vti_habc2_zeroobs", "vp", 1e-2), ("grad_rho_habc_zeroobs", "rho", 1e-2)]


def _misfit(g, models):
    out = fd2d.forward(g["equation"], models, g["d"], g["dt"], g["h"], g["wavelet"], g["sources"],
                       g["receivers"], order=g["order"], multiple=g["multiple"],
                       source_type=g["source_type"], receiver_type=g["receiver_type"])
    return float(sum(np.sum(r.astype(np.float64) ** 2) for r in out["records"]))


@pytest.mark.parametrize("name,param,step", CASES)
def test_gradient_golden_matches_oracle_finite_differences(name, param, step):
    g = load(name)
    grad = g["grad_" + param]
    w = g["width"]
    box = np.zeros_like(grad, bool)
    box[(0 if g["multiple"] else w):-w, w:-w] = True
    flat = np.argsort(np.where(box, np.abs(grad), 0.0).ravel())[-2:]  # two largest cells in the box
    for idx in flat:
        z, x = np.unravel_index(idx, grad.shape)
        plus = {k: v.copy() for k, v in g["models"].items()}
        minus = {k: v.copy() for k, v in g["models"].items()}
        plus[param][z, x] += step
        minus[param][z, x] -= step
        fd = (_misfit(g, plus) - _misfit(g, minus)) / (2 * step)
        assert abs(fd - grad[z, x]) < 1e-4 * abs(grad[z, x]), (param, z, x, fd, grad[z, x])
