"""Batched instances (uneven grids, one graph launch per step): the persistent multi-instance
step (one launch per phase for all instances) and the per-instance steps on several graph
streams give what the instances' own steps give one after another on one stream without a
graph (up to the order of the additions of the weight gradients, which is not fixed)."""

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


@pytest.mark.parametrize("arch,persistent", [((2, 16, 2, 16), True), ((2, 16, 2, 16), False), ((3, 32, 3, 32), True)])
def test_instance_batch_graph_matches_independent_steps(arch, persistent):
    arch = nn.Arch(*arch)
    insts = _instances()
    b = batch.InstanceBatch(insts, arch, batch=2048, lr=1e-3, seed=3, persistent=persistent).capture()
    assert b.persistent == persistent
    # same seeds, one instance after another, no graph
    ref = batch.InstanceBatch(insts, arch, batch=2048, lr=1e-3, seed=3, streams=1, persistent=False)
    for _ in range(4):
        lb = b.step().clone()
        lr = ref.step().clone()
    torch.cuda.synchronize()
    assert torch.isfinite(lb).all()
    np.testing.assert_allclose(lb.cpu().numpy(), lr.cpu().numpy(), rtol=1e-5)
    # the weight-gradient sums are added in another order; Adam (lr 1e-3) turns that into
    # parameter differences of a few 1e-7 on the smallest parameters
    for x, y in zip(b.items, ref.items):
        np.testing.assert_allclose(x.params.cpu().numpy(), y.params.cpu().numpy(), rtol=1e-4, atol=2e-6)
    assert b.points_per_step == sum(min(2048, it.level.n) for it in b.items)


def test_persistent_step_on_given_ids():
    """The persistent step on batch ids the caller put in place (ids_mode -1) against the
    per-instance steps on the same ids."""
    arch = nn.Arch(2, 16, 2, 16)
    insts = _instances()
    b = batch.InstanceBatch(insts, arch, batch=2048, lr=1e-3, seed=3)
    ref = batch.InstanceBatch(insts, arch, batch=2048, lr=1e-3, seed=3, persistent=False)
    rng = np.random.default_rng(11)
    for _ in range(3):
        for x, y in zip(b.items, ref.items):
            ids = torch.as_tensor(rng.choice(x.level.n, x.batch, replace=False).astype(np.int32), device="cuda")
            x.ids.copy_(ids)
            y.ids.copy_(ids)
        lb = b.step_with_ids().clone()
        lr = ref.step_with_ids().clone()
        np.testing.assert_allclose(lb.cpu().numpy(), lr.cpu().numpy(), rtol=1e-5)
    for x, y in zip(b.items, ref.items):
        np.testing.assert_allclose(x.params.cpu().numpy(), y.params.cpu().numpy(), rtol=1e-4, atol=2e-6)
