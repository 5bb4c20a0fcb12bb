"""The two non-C halves of the drop-in boundary, on the GPU.

* The XLA custom-call handlers ``dips_xla_loss_fwd`` / ``dips_xla_loss_bwd`` (what a
  jax.custom_vjp of ``Trainer.loss`` binds, solvers/poisson/trainer.py:892-912 and :783-789),
  called through ctypes the way XLA calls them: a ``void**`` buffer list (operands, then results,
  the workspace among the results), the descriptor bytes as ``opaque``, an opaque status.  They
  must give what ``dips_residual_fwd`` / ``dips_residual_bwd`` give.
* ``dips_gb300.ops.ResidualLoss``, the ``torch.autograd.Function`` that stands for
  ``value_and_grad(Trainer.loss)``: its loss and ``torch.autograd.grad`` against the oracle.
* The shapes whose kernels run a thread per job (1x1/2x10, 2x8) read their own call's weights:
  two parameter vectors on two streams, launched back to back without ordering, each give their
  own loss.
"""

import ctypes

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _xla_call(fn, bufs, desc, status=None):
    from dips_gb300 import _lib

    arr = (ctypes.c_void_p * len(bufs))(*[b.data_ptr() for b in bufs])
    fn(_lib.stream_handle(), arr, ctypes.cast(ctypes.byref(desc), ctypes.c_void_p), ctypes.sizeof(desc), status)


@pytest.mark.parametrize("arch", [(3, 32, 3, 32), (1, 1, 2, 10), (4, 64, 4, 64)])
def test_xla_handlers_match_the_residual_entry_points(arch):
    from dips_gb300 import _lib, ops

    lib = _lib.load()
    case = _parity.build_case("sphere", n=16, arch=arch, level=0, batch=1800, batch_seed=4)
    lvl = case.gpu_level()
    ga = case.gpu_arch()
    B = case.batch.size
    params = torch.as_tensor(case.params, device="cuda")
    ids = torch.as_tensor(case.batch, device="cuda")
    desc = _lib.XlaDescT()
    assert lib.dips_xla_make_desc(ga.ctype(), lvl.desc, B, lvl.max_jobs(B), ctypes.byref(desc)) == 0
    assert desc.ws_bytes == lib.dips_xla_workspace_bytes(ga.ctype(), B, lvl.max_jobs(B))

    loss = torch.full((), float("nan"), dtype=torch.float32, device="cuda")
    res = torch.empty(B, dtype=torch.float32, device="cuda")
    ws = torch.empty(desc.ws_bytes, dtype=torch.uint8, device="cuda")
    _xla_call(lib.dips_xla_loss_fwd, [params, ids, loss, res, ws], desc)
    g = torch.tensor(2.5, dtype=torch.float32, device="cuda")
    grad = torch.full((params.numel(),), float("nan"), dtype=torch.float32, device="cuda")
    ws2 = torch.empty(desc.ws_bytes, dtype=torch.uint8, device="cuda")
    _xla_call(lib.dips_xla_loss_bwd, [params, ids, g, grad, ws2], desc)

    l_ref, r_ref, wsr = ops.residual_forward(ga, params, lvl, ids, want_residual=True)
    g_ref = ops.residual_backward(ga, params, lvl, ids, wsr)
    torch.cuda.synchronize()
    assert abs(float(loss) - float(l_ref)) <= 1e-6 * abs(float(l_ref))
    np.testing.assert_array_equal(res.cpu().numpy(), r_ref.cpu().numpy())
    gr = 2.5 * g_ref.cpu().numpy().astype(np.float64)
    err = np.linalg.norm(grad.cpu().numpy() - gr) / np.linalg.norm(gr)
    assert err <= 1e-5, err


def test_xla_handler_failure_reaches_the_status():
    """A descriptor whose workspace result is too small: the handler launches nothing and the
    failure goes to the status setter (a Python stand-in for XlaCustomCallStatusSetFailure)."""
    from dips_gb300 import _lib

    lib = _lib.load()
    case = _parity.build_case("sphere", n=16, arch=(3, 32, 3, 32), batch=500, batch_seed=1)
    lvl = case.gpu_level()
    ga = case.gpu_arch()
    desc = _lib.XlaDescT()
    assert lib.dips_xla_make_desc(ga.ctype(), lvl.desc, 500, lvl.max_jobs(500), ctypes.byref(desc)) == 0
    desc.ws_bytes = 64
    seen = []

    @_lib.XlaStatusFn
    def setter(status, msg, n):
        seen.append((status, msg[:n].decode()))

    lib.dips_xla_set_status_fn(setter)
    try:
        params = torch.as_tensor(case.params, device="cuda")
        ids = torch.as_tensor(case.batch, device="cuda")
        loss = torch.full((), 7.0, dtype=torch.float32, device="cuda")
        res = torch.zeros(500, dtype=torch.float32, device="cuda")
        ws = torch.empty(64, dtype=torch.uint8, device="cuda")
        status = ctypes.create_string_buffer(32)
        _xla_call(lib.dips_xla_loss_fwd, [params, ids, loss, res, ws], desc, ctypes.cast(status, ctypes.c_void_p))
        torch.cuda.synchronize()
    finally:
        lib.dips_xla_set_status_fn(_lib.XlaStatusFn())
    assert len(seen) == 1 and seen[0][0] == ctypes.addressof(status) and "workspace" in seen[0][1]
    assert float(loss) == 7.0  # nothing ran


@pytest.mark.parametrize("arch", [(3, 32, 3, 32), (1, 1, 2, 10)])
def test_autograd_function_against_the_oracle(arch):
    from dips_gb300 import ops

    case = _parity.build_case("star", n=16, arch=arch, level=1, batch=2500, batch_seed=2)
    lvl = case.gpu_level()
    params = torch.as_tensor(case.params, device="cuda").requires_grad_(True)
    ids = torch.as_tensor(case.batch, device="cuda")
    loss = ops.residual_loss(params, case.gpu_arch(), lvl, ids)
    (grad,) = torch.autograd.grad(3.0 * loss, params)
    l_ref, g_ref = case.oracle_loss_grad()
    assert abs(float(loss) - float(l_ref)) <= 1e-5 * abs(float(l_ref))
    g = grad.cpu().numpy().astype(np.float64)
    gr = 3.0 * np.asarray(g_ref, np.float64)
    assert np.linalg.norm(g - gr) / np.linalg.norm(gr) <= 1e-4


@pytest.mark.parametrize("arch", [(1, 1, 2, 10), (2, 8, 2, 8)])
def test_per_job_kernels_read_their_own_calls_weights(arch):
    """Two parameter vectors, two streams, no ordering between the calls: each loss is the one
    its own parameters give alone."""
    from dips_gb300 import ops

    case = _parity.build_case("sphere", n=16, arch=arch, level=0)
    lvl = case.gpu_level()
    ga = case.gpu_arch()
    pa = torch.as_tensor(case.params, device="cuda")
    pb = torch.as_tensor(case.params * np.float32(-1.7) + np.float32(0.05), device="cuda")
    la0, _, wa = ops.residual_forward(ga, pa, lvl)
    lb0, _, wb = ops.residual_forward(ga, pb, lvl)
    torch.cuda.synchronize()
    assert abs(float(la0) - float(lb0)) > 1e-3 * abs(float(la0))
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    sa.wait_stream(torch.cuda.current_stream())
    sb.wait_stream(torch.cuda.current_stream())
    outs = []
    for _ in range(20):
        with torch.cuda.stream(sa):
            la, _, _ = ops.residual_forward(ga, pa, lvl, ws=wa)
        with torch.cuda.stream(sb):
            lb, _, _ = ops.residual_forward(ga, pb, lvl, ws=wb)
        outs.append((la, lb))
    torch.cuda.synchronize()
    for la, lb in outs:
        assert float(la) == float(la0) and float(lb) == float(lb0)
