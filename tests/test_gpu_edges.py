"""Edge cases of the batch path: ids outside the level, a batch whose jobs overflow the
workspace, one-point batches, repeated ids, and a batch of interface points only (no bulk tile).

Ids outside [0, n) and a job overflow are the cases the C ABI turns into NaN results rather
than errors (dips.h): the slot of a bad id gets a NaN residual and makes the loss NaN; an
overflow makes every residual NaN.  Neither may touch memory outside the workspace, and the
context stays usable.
"""

import numpy as np
import pytest
import torch

import _parity
from dips_gb300 import _lib, ops

pytestmark = pytest.mark.gpu
ARCH = (3, 32, 3, 32)


def _fwd(a, params, lvl, ids, ws):
    """dips_residual_fwd on the caller's workspace as given (ops.residual_forward would replace
    a workspace that is too small)."""
    lib = _lib.load()
    B = int(ids.numel())
    loss = torch.empty((), dtype=torch.float64, device="cuda")
    res = torch.empty(B, dtype=torch.float32, device="cuda")
    _lib.check(lib.dips_residual_fwd(a.ctype(), _lib.ptr(params), lvl.desc, _lib.ptr(ids), B, _lib.ptr(ws.buf),
                                     ws.nbytes, _lib.ptr(loss), _lib.ptr(res), _lib.stream_handle()),
               "dips_residual_fwd")
    torch.cuda.synchronize()
    return float(loss), res


def _case(arch=ARCH):
    case = _parity.build_case("sphere", n=16, arch=arch, level=0)
    return case, case.gpu_level(), case.gpu_arch(), torch.as_tensor(case.params, device="cuda")


@pytest.mark.parametrize("arch", [ARCH, (2, 16, 2, 16), (1, 1, 2, 10)])
def test_out_of_range_ids_give_nan_at_their_slots_only(arch):
    case, lvl, a, params = _case(arch)
    rng = np.random.default_rng(0)
    ids = torch.as_tensor(rng.choice(lvl.n, 500, replace=False).astype(np.int32), device="cuda")
    ws = ops.StepWorkspace(a, 500, lvl.max_jobs(500), "cuda")
    l0, r0 = _fwd(a, params, lvl, ids, ws)
    bad = ids.clone()
    bad[3] = lvl.n + 5
    bad[77] = -1
    l1, r1 = _fwd(a, params, lvl, bad, ws)
    assert np.isfinite(l0) and np.isnan(l1)
    assert torch.isnan(r1[3]) and torch.isnan(r1[77])
    keep = torch.ones(500, dtype=torch.bool, device="cuda")
    keep[3] = keep[77] = False
    assert torch.equal(r1[keep], r0[keep])


def test_job_overflow_gives_nan_and_leaves_the_context_usable():
    case, lvl, a, params = _case()
    ids = torch.arange(lvl.n, dtype=torch.int32, device="cuda")
    small = ops.StepWorkspace(a, lvl.n, 64, "cuda")  # room for 64 + slack jobs: the batch has thousands
    assert lvl.n_jobs > 10 * 64
    l1, r1 = _fwd(a, params, lvl, ids, small)
    assert np.isnan(l1) and torch.isnan(r1).all()
    ok = ops.StepWorkspace(a, lvl.n, lvl.max_jobs(lvl.n), "cuda")
    l2, r2 = _fwd(a, params, lvl, ids, ok)
    assert np.isfinite(l2) and torch.isfinite(r2).all()


def test_one_point_batches_bulk_and_interface():
    case, lvl, a, params = _case()
    ref = case.oracle_residual()  # every point, in id order
    cnt = lvl.cnt.cpu().numpy()
    bulk = int(np.nonzero(cnt == 7)[0][5])
    iface = int(np.nonzero(cnt > 7)[0][3])
    ws = ops.StepWorkspace(a, 1, lvl.max_cnt, "cuda")
    for pid in (bulk, iface):
        ids = torch.tensor([pid], dtype=torch.int32, device="cuda")
        loss, res = _fwd(a, params, lvl, ids, ws)
        assert abs(float(res[0]) - ref[pid]) <= 1e-5 * max(1.0, abs(ref[pid])), (pid, float(res[0]), ref[pid])
        assert abs(loss - 0.5 * float(res[0]) ** 2) <= 1e-6 * max(loss, 1e-30)


def test_repeated_ids_count_once_per_slot():
    case, lvl, a, params = _case()
    ref = case.oracle_residual()
    cnt = lvl.cnt.cpu().numpy()
    iface = int(np.nonzero(cnt > 7)[0][0])
    pids = [5, 5, 5, iface, iface, 900]
    ids = torch.tensor(pids, dtype=torch.int32, device="cuda")
    ws = ops.StepWorkspace(a, len(pids), lvl.max_jobs(len(pids), distinct=False), "cuda")
    loss, res = _fwd(a, params, lvl, ids, ws)
    r = res.cpu().numpy()
    assert r[0] == r[1] == r[2] and r[3] == r[4]
    np.testing.assert_allclose(r, ref[pids], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(loss, np.mean(0.5 * r.astype(np.float64) ** 2), rtol=1e-6)


def test_interface_only_batch_has_no_bulk_tile():
    """Every point of the batch is general (its residual needs cube-vertex jobs): no bulk tile,
    general tiles only, and the loss and gradient still match the oracle."""
    case, lvl, a, params = _case()
    cnt = lvl.cnt.cpu().numpy()
    case.batch = np.nonzero(cnt > 7)[0].astype(np.int32)
    case._rg = None
    assert case.batch.size > 100
    lg, gg = case.gpu_loss_grad()
    lo, go = case.oracle_loss_grad()
    assert abs(lg - lo) <= 1e-5 * abs(lo)
    assert np.linalg.norm(gg - go) <= 1e-4 * np.linalg.norm(go)
