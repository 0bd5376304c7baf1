"""Multi-rank path on CPU (gloo, world size 2): shots are sharded across the
ranks and the per-rank gradients are summed by one all-reduce.  Each rank
computes its shard's gradient with the oracle (the GPU kernels are not
available here); the reduced gradient must equal the single-process gradient
over all shots."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from tests.golden_cases import load


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    from oracle import adjoint
    from seistorch_gb300.distributed import allreduce_gradient, reduce_loss, shard_shots
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = load("grad_acoustic_pml_o4_zeroobs")
    mine = shard_shots(range(len(g["sources"])), rank, world)
    resid = [2.0 * g["records"][b] for b in mine]
    grad = adjoint.acoustic_pml_gradient(g["models"]["vp"], g["d"], g["dt"], g["h"], g["wavelet"],
                                         [g["sources"][b] for b in mine], [g["receivers"][b] for b in mine],
                                         resid, order=g["order"])
    t = torch.tensor(grad)
    allreduce_gradient(t)
    loss = reduce_loss(float(sum(np.sum(g["records"][b] ** 2) for b in mine)))
    if rank == 0:
        np.savez(out_path, grad=t.numpy(), loss=float(loss))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_shots_covers_every_shot_once():
    from seistorch_gb300.distributed import shard_shots
    for n in (0, 1, 5, 64):
        for w in (1, 2, 3, 8):
            parts = [shard_shots(range(n), r, w) for r in range(w)]
            assert sum(parts, []) == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        shard_shots(range(4), 2, 2)


def test_two_gloo_ranks_sum_to_the_single_process_gradient(tmp_path):
    out = str(tmp_path / "r0.npz")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    from oracle import adjoint
    g = load("grad_acoustic_pml_o4_zeroobs")
    want = adjoint.acoustic_pml_gradient(g["models"]["vp"], g["d"], g["dt"], g["h"], g["wavelet"], g["sources"],
                                         g["receivers"], [2.0 * r for r in g["records"]], order=g["order"])
    got = np.load(out)
    np.testing.assert_allclose(got["grad"], want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    assert abs(float(got["loss"]) - float(g["loss"])) < 1e-9 * float(g["loss"])
