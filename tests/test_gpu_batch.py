"""Batched instances (uneven grids, one graph launch per step, instances side by side on the
graph's streams): every instance's step in the captured graph gives what the same step gives
when the instances run one after another on one stream without a graph (up to the order of the
shared-memory atomic additions of the weight gradients, which is not fixed)."""

import numpy as np
import pytest
import torch

from dips_gb300 import batch, nn, ops, problems

pytestmark = pytest.mark.gpu


def _instances():
    out = []
    for side, c, r, q in problems.lpbe_instances(3, seed=4):
        side = [16, 24, 32][len(out)]
        k = min(len(c), 60)
        out.append((side, problems.lpbe_problem(c[:k], r[:k], q[:k])))
    return out


def test_instance_batch_graph_matches_independent_steps():
    arch = nn.Arch(2, 16, 2, 16)
    insts = _instances()
    b = batch.InstanceBatch(insts, arch, batch=2048, lr=1e-3, seed=3).capture()
    ref = batch.InstanceBatch(insts, arch, batch=2048, lr=1e-3, seed=3, streams=1)  # same seeds, no graph
    for _ in range(4):
        lb = b.step().clone()
        lr = ref.step().clone()
    torch.cuda.synchronize()
    assert torch.isfinite(lb).all()
    np.testing.assert_allclose(lb.cpu().numpy(), lr.cpu().numpy(), rtol=1e-5)
    for x, y in zip(b.items, ref.items):
        np.testing.assert_allclose(x.params.cpu().numpy(), y.params.cpu().numpy(), rtol=1e-4, atol=1e-7)
    assert b.points_per_step == sum(min(2048, it.level.n) for it in b.items)
