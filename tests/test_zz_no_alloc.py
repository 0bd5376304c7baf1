"""The allocation-free adjoint entry point (sgb_acoustic_backward_noalloc).

It serves callers that cannot allocate device memory themselves -- a host
application or plugin framework that owns all device memory and forbids
cudaMalloc/cudaFree on its threads, or a loop that must not allocate while it
runs -- by keeping the adjoint's scratch in a fixed device array inside the
library.  Two calls in a row through the C ABI must give the gradient of the
regular entry point (which takes caller-allocated scratch) within the
gradient tolerance of the other tests (relative L2 1e-4); the second call
also shows that what the first call left in the shared array does not leak
into the next, and the device's free memory (cudaMemGetInfo) is the same
before and after it: the call allocates nothing.  This file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests.golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu


def _forward_state(g, dev, prop, acq):
    vp = torch.tensor(g["models"]["vp"], dtype=torch.float32, device=dev)
    d = torch.tensor(g["d"], dtype=torch.float32, device=dev)
    rec, state, _ = prop.forward(vp, d, acq, save_for_adjoint=True, ckpt_every=25)
    return rec, state


def test_noalloc_adjoint_matches_allocating_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from seistorch_gb300 import _native as N
    from seistorch_gb300 import engine
    N.load(build_if_missing=False)
    dev = torch.device("cuda:0")
    g = load("grad_acoustic_pml_o4_zeroobs")
    nz, nx = g["models"]["vp"].shape
    prop = engine.AcousticPropagator(nz, nx, g["dt"], g["h"], g["order"], "pml", g["width"], False, dev)
    acq = engine.Acquisition(nz, nx, g["sources"], g["receivers"], g["wavelet"], dev)

    rec, state = _forward_state(g, dev, prop, acq)
    resid = (2.0 * rec).contiguous()
    want = prop.backward(state, acq, resid).cpu().numpy()
    assert np.isfinite(want).all() and np.abs(want).max() > 0

    for call in range(2):
        rec, state = _forward_state(g, dev, prop, acq)
        resid = (2.0 * rec).contiguous()
        res = torch.zeros(acq.nt, acq.nrec, 1, dtype=torch.float32, device=dev)
        res[:] = resid.reshape(acq.nt, acq.nrec, 1)
        grad = torch.empty(nz, prop.pitch, dtype=torch.float32, device=dev)
        gr = prop.grid(acq.nshots)
        q = acq.struct(res, 1)
        ub = N.PTR3(*[b.data_ptr() for b in state.buf])
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        N.call("sgb_acoustic_backward_noalloc", ctypes.byref(gr), ctypes.byref(state.model), ctypes.byref(q),
               ctypes.byref(state.bs), ub, state.cur, state.prev, N.ptr(grad), N.stream_handle())
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        if call == 1:  # the first call may load the kernels' module; the second must not allocate
            assert free_after == free_before, (free_before, free_after)
        got = grad[:, :nx].cpu().numpy()
        assert rel_l2(got, want) < 1e-4


def test_noalloc_adjoint_rejects_problems_beyond_its_scratch():
    from seistorch_gb300 import _native as N
    lib = N.load(build_if_missing=False)
    # 64 shots x 500 x 1100: 4 fields exceed the 8 Mi-float scratch
    gr = N.Grid(500, 1100, 1100, 64, 0.001, 10.0)
    status = lib.sgb_acoustic_backward_noalloc(ctypes.byref(gr), None, None, None, N.PTR3(), 0, 1, None, None)
    assert status == 8
    assert b"scratch" in lib.sgb_status_string(status)
