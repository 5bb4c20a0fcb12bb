"""dips_train_step_noalloc (the training step whose scratch is the library's built-in
device array, for callers that cannot allocate device memory) must give the same step as
dips_train_step with a caller-allocated workspace, on two calls in a row.  Collected last
(file name) so that a run stopping at the first failure has run every other test first."""

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_noalloc_step_matches_workspace_step_twice():
    from dips_gb300 import _lib, ops

    lib = _lib.load()
    case = _parity.build_case("sphere", n=16, arch=(3, 32, 3, 32), level=1)
    lvl = case.gpu_level()
    arch = case.gpu_arch()
    P = case.params.size
    B = 1500
    ids = torch.as_tensor(np.random.default_rng(2).choice(lvl.n, B, replace=False).astype(np.int32), device="cuda")
    max_jobs = lvl.max_jobs(B)

    # A: existing entry point with a caller-allocated workspace
    pa = torch.as_tensor(case.params.copy(), device="cuda")
    oa = ops.AdamState(P, lr=1e-3, decay_rate=0.9)
    ws = ops.StepWorkspace(arch, B, max_jobs)
    la = torch.empty((), dtype=torch.float64, device="cuda")
    ga = torch.empty(P, dtype=torch.float32, device="cuda")
    # B: the no-allocation entry point through the C ABI
    pb = torch.as_tensor(case.params.copy(), device="cuda")
    ob = ops.AdamState(P, lr=1e-3, decay_rate=0.9)
    lb = torch.empty((), dtype=torch.float64, device="cuda")
    gb = torch.empty(P, dtype=torch.float32, device="cuda")
    st = _lib.stream_handle()
    for _ in range(2):
        ops.train_step(arch, pa, oa, lvl, ids, ws, la, ga)
        status = lib.dips_train_step_noalloc(arch.ctype(), ob.hp, _lib.ptr(pb), _lib.ptr(ob.mu), _lib.ptr(ob.nu),
                                             _lib.ptr(ob.count), lvl.desc, _lib.ptr(ids), B, max_jobs, _lib.ptr(lb),
                                             _lib.ptr(gb), st)
        assert status == 0, lib.dips_last_error()
        torch.cuda.synchronize()
        assert abs(float(lb) - float(la)) <= 1e-5 * abs(float(la))
        g_a, g_b = ga.cpu().numpy(), gb.cpu().numpy()
        assert np.linalg.norm(g_b - g_a) <= 1e-4 * np.linalg.norm(g_a)
        np.testing.assert_allclose(pb.cpu().numpy(), pa.cpu().numpy(), rtol=1e-5, atol=1e-7)
    assert int(ob.count.item()) == 2


def test_noalloc_rejects_oversized_batches():
    from dips_gb300 import _lib, ops

    lib = _lib.load()
    case = _parity.build_case("sphere", n=16, arch=(3, 32, 3, 32))
    lvl = case.gpu_level()
    arch = case.gpu_arch()
    P = case.params.size
    p = torch.as_tensor(case.params.copy(), device="cuda")
    o = ops.AdamState(P)
    loss = torch.empty((), dtype=torch.float64, device="cuda")
    status = lib.dips_train_step_noalloc(arch.ctype(), o.hp, _lib.ptr(p), _lib.ptr(o.mu), _lib.ptr(o.nu),
                                         _lib.ptr(o.count), lvl.desc, None, lvl.n, 10**9, _lib.ptr(loss), None,
                                         _lib.stream_handle())
    assert status == 3 and b"built-in" in lib.dips_last_error()
    assert int(o.count.item()) == 0
