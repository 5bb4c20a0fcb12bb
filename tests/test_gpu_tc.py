"""The 4x64 DoubleMLP on the tensor cores (tcgen05.mma kind::tf32, FP32 accumulation in TMEM).

TF32 operands carry 10 mantissa bits, so the bars are stated against the FP64 oracle. The loss
must agree to 1e-5 relative, because the forward's rounding averages out over the batch. The
gradient must agree to 1e-3 relative in the L2 norm; measured errors are about 1.5e-4 against
2e-7 for the FP32 oracle.
"""

import numpy as np
import pytest
import torch

import _parity
from dips_gb300 import nn

pytestmark = pytest.mark.gpu

ARCH = (4, 64, 4, 64)


@pytest.mark.parametrize("name,n,level", [("sphere", 12, 0), ("sphere", 16, 1), ("star", 16, 0)])
def test_tf32_loss_and_gradient_against_fp64(name, n, level):
    case = _parity.build_case(name, n=n, arch=ARCH, level=level)
    lg, gg = case.gpu_loss_grad()
    l64, g64 = case.oracle_loss_grad(torch.float64)
    gg = np.asarray(gg, np.float64)
    g64 = np.asarray(g64, np.float64)
    assert np.isfinite(lg) and np.isfinite(gg).all()
    assert abs(lg - l64) <= 1e-5 * abs(l64), (lg, l64)
    err = np.linalg.norm(gg - g64) / np.linalg.norm(g64)
    assert err <= 1e-3, err
    # every parameter block receives its gradient (W1, b1, W2..W4, b2..b4, w_o, b_o of both nets)
    a = nn.Arch(*ARCH)
    blocks = np.split(g64, np.cumsum(_block_sizes(a))[:-1])
    gblocks = np.split(gg, np.cumsum(_block_sizes(a))[:-1])
    gnorm = np.linalg.norm(g64)
    for k, (b64, bg) in enumerate(zip(blocks, gblocks)):
        nb = np.linalg.norm(b64)
        if nb > 1e-3 * gnorm:  # blocks that carry a visible share of the gradient
            rel = np.linalg.norm(bg - b64) / nb
            assert rel <= 2e-2, (k, b64.size, rel, nb / gnorm)


def _block_sizes(a):
    sizes = []
    for which in ("m", "p"):
        L, W = a.net(which)
        sizes += [3 * W, W]
        for _ in range(L - 1):
            sizes += [W * W, W]
        sizes += [W, 1]
    return sizes


def test_tf32_train_steps_reduce_the_loss():
    case = _parity.build_case("sphere", n=16, arch=ARCH, level=0)
    from dips_gb300 import ops

    lvl = case.gpu_level()
    a = nn.Arch(*ARCH)
    params = torch.as_tensor(case.params, device="cuda")
    opt = ops.AdamState(nn.n_params(a), lr=1e-3, decay_rate=0.9)
    ws = ops.StepWorkspace(a, lvl.n, lvl.max_jobs(lvl.n), "cuda")
    loss = torch.zeros((), dtype=torch.float64, device="cuda")
    losses = []
    for _ in range(30):
        ops.train_step(a, params, opt, lvl, None, ws, loss)
        losses.append(float(loss))
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.5 * losses[0], losses


def test_mlp_eval_4x64():
    case = _parity.build_case("star", n=12, arch=ARCH, level=0)
    L = _parity.L
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1, 1, (3000, 3)).astype(np.float32)
    phi = case.oracle_problem.phi(pts)
    u, g = nn.mlp_eval(case.gpu_arch(), torch.as_tensor(case.params, device="cuda"),
                       torch.as_tensor(pts, device="cuda"), torch.as_tensor(phi, device="cuda"), want_grad=True)
    x = torch.tensor(pts, dtype=torch.float64, requires_grad=True)
    ref = L.nn_eval(L.unflatten(torch.tensor(case.params, dtype=torch.float64), case.arch), x, phi)
    (gref,) = torch.autograd.grad(ref.sum(), x)
    np.testing.assert_allclose(u.cpu().numpy(), ref.detach().numpy(), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(g.cpu().numpy(), gref.numpy(), rtol=1e-4, atol=1e-5)


def test_wait_timeout_gives_nan_and_the_next_call_is_clean():
    """The bounded mbarrier waits, made to run out: with a limit of 0 polls every wait gives up at
    once (the MMAs it waited for still complete).  The call must report it -- loss and gradient
    NaN -- after each CTA waited for its MMAs in flight and freed its tensor memory; the next call
    at the default limit must give the normal result (an allocation left behind would stall it)."""
    from dips_gb300 import _lib, ops

    lib = _lib.load()
    case = _parity.build_case("sphere", n=12, arch=ARCH, level=0)
    lvl = case.gpu_level()
    a = case.gpu_arch()
    params = torch.as_tensor(case.params, device="cuda")
    l0, _, ws = ops.residual_forward(a, params, lvl)
    g0 = ops.residual_backward(a, params, lvl, None, ws)
    torch.cuda.synchronize()
    old = lib.dips_tc_set_wait_limit(0)
    try:
        l1, _, ws = ops.residual_forward(a, params, lvl, ws=ws)
        g1 = ops.residual_backward(a, params, lvl, None, ws)
        torch.cuda.synchronize()
    finally:
        assert lib.dips_tc_set_wait_limit(old) == 0
    assert old == 1 << 24
    assert np.isnan(float(l1)) and torch.isnan(g1).all()
    l2, _, ws = ops.residual_forward(a, params, lvl, ws=ws)
    g2 = ops.residual_backward(a, params, lvl, None, ws)
    torch.cuda.synchronize()
    assert float(l2) == float(l0)
    np.testing.assert_allclose(g2.cpu().numpy(), g0.cpu().numpy(), rtol=1e-5, atol=1e-7)
