"""Checkpoint format and restart (solvers/poisson/trainer.py:326-351 and :255-263) on the CPU.
Trainer.save_checkpoint and Trainer._restore touch only host copies of the parameters and of
the optimizer state, so they run here on a stand-in that holds the attributes they read."""

import os
import pickle
import types

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from dips_gb300 import nn  # noqa: E402
from dips_gb300.trainer import Trainer  # noqa: E402

ARCH = nn.Arch(1, 1, 2, 10)


def _trainer(seed, count, num_epochs=200):
    rng = np.random.default_rng(seed)
    P = nn.n_params(ARCH)
    opt = types.SimpleNamespace(mu=torch.as_tensor(rng.standard_normal(P).astype(np.float32)),
                                nu=torch.as_tensor(rng.random(P).astype(np.float32)),
                                count=torch.tensor(count, dtype=torch.int64))
    return types.SimpleNamespace(params=torch.as_tensor(nn.init_params(ARCH, seed)), opt=opt, arch=ARCH,
                                 batch=4096, h0=(0.0625, 0.0625, 0.0625), device="cpu", num_epochs=num_epochs,
                                 epoch_start=0)


def test_checkpoint_contents_follow_the_reference_format(tmp_path):
    t = _trainer(1, 17)
    path = Trainer.save_checkpoint(t, str(tmp_path), 25)
    assert os.path.basename(path) == "checkpoint_25"
    with open(path, "rb") as f:
        state = pickle.load(f)
    assert set(state) == {"opt_state", "params", "epoch", "batch_size", "resolution"}
    assert state["epoch"] == 25 and state["batch_size"] == 4096
    assert state["resolution"] == "0.0625, 0.0625, 0.0625"
    assert state["opt_state"]["count"] == 17
    tree = state["params"]
    assert any("_m_fn" in k for k in tree) and any("_p_fn" in k for k in tree) and tree["preconditioner"] == {}
    np.testing.assert_array_equal(nn.tree_to_params(tree, ARCH).numpy(), t.params.numpy())


def test_restore_takes_the_highest_epoch_numerically(tmp_path):
    saved = {}
    for epoch in (9, 10, 100):  # by string order "checkpoint_9" would be the last
        t = _trainer(epoch, epoch * 3)
        Trainer.save_checkpoint(t, str(tmp_path), epoch)
        saved[epoch] = t
    for num_epochs, start in ((200, 100), (50, 50)):
        r = _trainer(0, 0, num_epochs=num_epochs)
        Trainer._restore(r, str(tmp_path))
        want = saved[100]
        np.testing.assert_array_equal(r.params.numpy(), want.params.numpy())
        np.testing.assert_array_equal(r.opt.mu.numpy(), want.opt.mu.numpy())
        np.testing.assert_array_equal(r.opt.nu.numpy(), want.opt.nu.numpy())
        assert int(r.opt.count) == 300
        assert r.epoch_start == start


def test_restore_without_checkpoints_changes_nothing(tmp_path):
    t = _trainer(3, 5)
    before = t.params.clone()
    Trainer._restore(t, str(tmp_path / "missing"))
    Trainer._restore(t, str(tmp_path))
    Trainer._restore(t, "")
    assert torch.equal(t.params, before) and int(t.opt.count) == 5 and t.epoch_start == 0


def test_restore_skips_stray_files_and_refuses_another_batch_size(tmp_path):
    t = _trainer(4, 12)
    Trainer.save_checkpoint(t, str(tmp_path), 40)
    for stray in ("checkpoint_100.tmp", "checkpoint_90.bak", "checkpoint_final"):
        (tmp_path / stray).write_bytes(b"not a pickle")
    r = _trainer(0, 0)
    Trainer._restore(r, str(tmp_path))
    np.testing.assert_array_equal(r.params.numpy(), t.params.numpy())
    assert r.epoch_start == 40 and int(r.opt.count) == 12
    other = _trainer(0, 0)
    other.batch = 2048
    with pytest.raises(ValueError, match="batch_size 4096"):
        Trainer._restore(other, str(tmp_path))
    assert int(other.opt.count) == 0


def test_interval_checkpoints_of_the_multi_gpu_loop(tmp_path):
    """multi_GPU_train saves after every checkpoint_interval-th epoch (trainer.py:769-777); one
    rank writes (the ranks hold the same state); the single-GPU loop saves at the end only."""
    d = str(tmp_path)
    t = _trainer(3, 5)
    t.checkpoint_dir, t.checkpoint_interval = d, 4
    t.save_checkpoint = lambda cdir, epoch: Trainer.save_checkpoint(t, cdir, epoch)
    for multi, rank in ((False, 0), (True, 1)):
        t.multi_gpu, t.rank = multi, rank
        assert all(Trainer._interval_checkpoint(t, e) is None for e in range(12))
    assert os.listdir(d) == []
    t.multi_gpu, t.rank = True, 0
    written = [Trainer._interval_checkpoint(t, e) for e in range(12)]
    assert [os.path.basename(p) for p in written if p] == ["checkpoint_4", "checkpoint_8", "checkpoint_12"]
    t.checkpoint_interval = 0
    assert Trainer._interval_checkpoint(t, 15) is None
    r = _trainer(0, 0)
    Trainer._restore(r, d)
    assert r.epoch_start == 12
