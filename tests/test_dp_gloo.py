"""Data-parallel training step on two CPU processes (gloo): the per-device batch layout of
DatasetDict(num_gpus=2) and the psum of gradient and loss (solvers/poisson/trainer.py:716-834).

Each rank evaluates the oracle's loss and gradient on its own batch, the gradients and losses
are summed across ranks with dips_gb300.dp, and both ranks apply the same Adam update.  The
checks: the device batches partition the points, the reduced gradient equals the sum of the
per-device gradients computed serially, and the two ranks end with identical parameters.
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import _parity
from dips_gb300 import dp

L = _parity.L
O = _parity.O


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_device_batches_layout():
    # 10 points on 3 devices, batch 4: runs of 4, the last device gets 2 points + 2 padding
    bs, lay = dp.device_batches(10, 4, 3)
    assert bs == 4
    assert lay == [[(0, 4, 0)], [(4, 8, 0)], [(8, 10, 2)]]
    # 10 points on 2 devices, batch 3: one full batch and one padded extra batch each
    bs, lay = dp.device_batches(10, 3, 2)
    assert bs == 3 and lay == [[(0, 3, 0), (3, 5, 1)], [(5, 8, 0), (8, 10, 1)]]
    # every point in exactly one batch
    for n, b, g in [(1000, 64, 2), (1000, 1000, 4), (4096, 512, 8), (777, 50, 3)]:
        _, lay = dp.device_batches(n, b, g)
        seen = np.zeros(n, np.int32)
        for rows in lay:
            for begin, end, _ in rows:
                seen[begin:end] += 1
        assert (seen == 1).all()


def _case():
    case = _parity.Case("sphere", n=10, arch=(1, 1, 2, 10), level=0)
    return case, case.oracle_problem


def _grad_on(case, prob, pts):
    rg = L.ResidualGeometry(prob, pts, case.h)
    loss, grad = L.loss_and_grad(case.params, case.arch, rg)
    return float(loss), np.asarray(grad, np.float32)


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        case, prob = _case()
        pts = np.asarray(case.pts, np.float32)
        # the reference passes batch_size = n_devices * batch_size to DatasetDict (trainer.py:733-737)
        batch = 256
        mine, bs, nb = dp.device_points(pts, world * batch, rank, world, lambda c: pts[:c])
        first = mine[:bs]
        loss, grad = _grad_on(case, prob, first)
        g = torch.tensor(grad)
        lo = torch.tensor([loss], dtype=torch.float64)
        dp.allreduce_sum_(g, lo)
        opt = O.ChainedAdam(g.numel(), lr=1e-2)
        new = opt.update(case.params.copy(), g.numpy())
        out[rank] = (g.numpy().copy(), float(lo), np.asarray(new, np.float32), bs, nb)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(600)
def test_two_rank_gradient_sum_and_update():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    case, prob = _case()
    pts = np.asarray(case.pts, np.float32)
    ref_g = 0.0
    ref_l = 0.0
    for r in range(world):
        mine, bs, _ = dp.device_points(pts, world * 256, r, world, lambda c: pts[:c])
        l, g = _grad_on(case, prob, mine[:bs])
        ref_g = ref_g + g
        ref_l += l
    for r in range(world):
        g, lo, new, _, _ = res[r]
        # float32 sums in the ranks' processes may use another thread split than this one's
        np.testing.assert_allclose(g, ref_g, rtol=1e-5, atol=1e-8)
        assert abs(lo - ref_l) <= 1e-6 * abs(ref_l)
    np.testing.assert_array_equal(res[0][2], res[1][2])  # both ranks apply the same update
