"""Shot sharding and the per-iteration gradient all-reduce on two gloo ranks (CPU).

Each rank computes the gradient of its round-robin shard with the CPU oracle
(the per-GPU compute is stood in by the checker here; the GPU plan is tested
on its own) and the all-reduced result must equal the serial sum over all
shots."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _case():
    rng = np.random.default_rng(0)
    NX, NY, T = 16, 12, 30
    vp = 2000 + 300 * rng.random((NX + 2) * (NY + 2))
    shots = [dict(srci=[3 + 3 * k], srcj=[4], srcv=rng.standard_normal((T, 1)) * 100,
                  rcvi=np.arange(2, 16), rcvj=np.full(14, 3)) for k in range(5)]
    obs = [rng.standard_normal((T + 1, 14)) * 1e-4 for _ in shots]
    return NX, NY, T, vp, shots, obs


def _grad(orc, NX, NY, T, vp, shot, obs):
    sx, ty = orc.acoustic_pml(NX, NY, 10.0, 10.0, 4, 2000.0)
    return orc.acoustic_gradient(NX, NY, T, 1e-3, 10.0, 10.0, sx, ty, vp, shot["srci"],
                                 shot["srcj"], shot["srcv"], shot["rcvi"], shot["rcvj"], obs)


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import __graft_entry__ as g
    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ads = g.load_package()
    from adseismic_gb300.distributed import allreduce_loss_grad, shard_shots

    NX, NY, T, vp, shots, obs = _case()
    mine = shard_shots(list(zip(shots, obs)), rank, world)
    loss = torch.zeros(1, dtype=torch.float64)
    grad = torch.zeros(vp.size, dtype=torch.float64)
    for shot, o in mine:
        l, gr = _grad(oracle, NX, NY, T, vp, shot, o)
        loss += l
        grad += torch.from_numpy(gr)
    allreduce_loss_grad(loss, grad)
    out[rank] = (float(loss), grad.numpy().copy())
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_shard_round_robin(ads):
    from adseismic_gb300.distributed import shard_shots

    assert shard_shots(list(range(7)), 1, 3) == [1, 4]
    assert sum(len(shard_shots(list(range(7)), r, 3)) for r in range(3)) == 7
    with pytest.raises(ValueError):
        shard_shots([1], 2, 2)


def test_two_rank_gradient_sum_equals_serial(orc):
    NX, NY, T, vp, shots, obs = _case()
    ref_loss, ref_grad = 0.0, np.zeros(vp.size)
    for s, o in zip(shots, obs):
        l, g = _grad(orc, NX, NY, T, vp, s, o)
        ref_loss += l
        ref_grad += g
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        loss, grad = out[r]
        assert loss == pytest.approx(ref_loss, rel=1e-13)
        assert np.allclose(grad, ref_grad, rtol=1e-12, atol=1e-30)
