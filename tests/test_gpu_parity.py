"""CUDA path vs the CPU oracle, through the C ABI.

Bars: integer/flag outputs and the level-set interpolant bit-exact; geometry
coefficients bit-exact where the coefficient callables are constants (the float32
operations are the oracle's, with no FMA contraction); loss within 1e-5 relative and
gradients within 1e-4 relative (the tolerances required of the FP32 path).
"""

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

O = _parity.O
L = _parity.L
F32 = np.float32

LOSS_RTOL = 1e-5
GRAD_RTOL = 1e-4


def _grad_close(g, ref):
    err = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    assert err < GRAD_RTOL, f"gradient rel err {err:.3e}"
    # componentwise, relative to the largest component
    assert np.max(np.abs(g - ref)) <= GRAD_RTOL * np.max(np.abs(ref)) * 10


def test_ghost_layer_and_trilinear_bit_exact():
    from dips_gb300 import levelset

    case = _parity.build_case("star", n=20)
    ls = levelset.LevelSetGrid(case.grid, case.phi)
    T = O.Trilinear(case.phi, case.grid.x, case.grid.y, case.grid.z)
    np.testing.assert_array_equal(ls.gh.cpu().numpy().reshape(T.gh.shape), T.gh)
    rng = np.random.default_rng(3)
    pts = rng.uniform(-1.3, 1.3, (20000, 3)).astype(F32)
    pts[:50] = case.grid.R[rng.choice(case.grid.R.shape[0], 50)]  # grid nodes, incl. the first cell
    pts[50:60, 0] = case.grid.x[0]
    pts[60:70, 1] = case.grid.y[-1]
    got = ls(torch.as_tensor(pts, device="cuda")).cpu().numpy()
    np.testing.assert_array_equal(got, T(pts))


@pytest.mark.parametrize("level", [0, 1, 2])
def test_geometry_flags_and_coefficients(level):
    case = _parity.build_case("sphere", n=24, level=level)
    lvl = case.gpu_level()
    rg = case.oracle_geometry()
    f = lvl.flags.cpu().numpy().astype(np.uint32)
    bnd = (f & 1).astype(bool)
    np.testing.assert_array_equal(bnd, rg.bnd)
    cp = ((f >> 1) & 3).astype(np.int64) - 1
    np.testing.assert_array_equal(cp, rg.crossed_p.astype(np.int64))
    for j in range(7):
        cs = ((f >> (4 + 2 * j)) & 3).astype(np.int64) - 1
        np.testing.assert_array_equal(cs, rg.crossed_s[:, j].astype(np.int64), err_msg=f"stencil {j}")
        net = ((f >> (18 + j)) & 1).astype(bool)
        np.testing.assert_array_equal(net, rg.phi_s[:, j] >= 0)
    np.testing.assert_array_equal(lvl.coeff26.cpu().numpy(), rg.coeffs)
    np.testing.assert_allclose(lvl.beta_int.cpu().numpy(), rg.beta_int, rtol=2e-6, atol=1e-9)
    assert int(lvl.n_xs.sum()) == int((rg.crossed_s[~rg.bnd] == 0).sum())


@pytest.mark.parametrize(
    "name,n,arch,level",
    [
        ("sphere", 16, (1, 1, 2, 10), 0),
        ("sphere", 24, (1, 1, 2, 10), 1),
        ("sphere", 16, (1, 1, 2, 10), 3),
        ("star", 20, (2, 8, 2, 8), 0),
        ("star", 20, (2, 16, 2, 16), 1),
        ("sphere", 20, (3, 32, 3, 32), 0),
        ("star", 16, (3, 32, 3, 32), 2),
    ],
)
def test_loss_and_gradient(name, n, arch, level):
    case = _parity.build_case(name, n=n, arch=arch, level=level)
    lg, gg = case.gpu_loss_grad()
    lr, gr = case.oracle_loss_grad()
    assert abs(lg - lr) <= LOSS_RTOL * abs(lr), (lg, lr)
    _grad_close(gg, gr)
    # the oracle's own FP32 error against FP64 is far below the bars
    l64, g64 = case.oracle_loss_grad(torch.float64)
    assert abs(lr - l64) <= 1e-6 * abs(l64)


def test_residual_vector_and_minibatch():
    case = _parity.build_case("star", n=24, arch=(2, 16, 2, 16), level=1, batch=3000, batch_seed=5)
    r_gpu = case.gpu_residual()
    r_ref = case.oracle_residual()
    scale = np.max(np.abs(r_ref))
    np.testing.assert_allclose(r_gpu, r_ref, rtol=1e-4, atol=1e-5 * scale)
    lg, gg = case.gpu_loss_grad()
    lr, gr = case.oracle_loss_grad()
    assert abs(lg - lr) <= LOSS_RTOL * abs(lr)
    _grad_close(gg, gr)


@pytest.mark.parametrize("arch", [(3, 32, 3, 32), (2, 16, 2, 16), (1, 1, 2, 10)])
def test_mlp_eval_and_input_gradient(arch):
    """u and du/dx (the tile engine's evaluation for 3x32 and 2x16, a thread per point for the
    other shapes) against the oracle's network in FP64 with autograd; 5,001 points, so that the
    last 32-point tile is partial and most tiles straddle the interface."""
    from dips_gb300 import nn

    case = _parity.build_case("sphere", n=16, arch=arch)
    rng = np.random.default_rng(0)
    pts = rng.uniform(-1, 1, (5001, 3)).astype(F32)
    phi = case.oracle_problem.phi(pts)
    u, g = nn.mlp_eval(case.gpu_arch(), torch.as_tensor(case.params, device="cuda"),
                       torch.as_tensor(pts, device="cuda"), torch.as_tensor(phi, device="cuda"), want_grad=True)
    x = torch.tensor(pts, dtype=torch.float64, requires_grad=True)
    net = L.unflatten(torch.tensor(case.params, dtype=torch.float64), case.arch)
    ref = L.nn_eval(net, x, phi)
    (gref,) = torch.autograd.grad(ref.sum(), x)
    np.testing.assert_allclose(u.cpu().numpy(), ref.detach().numpy(), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(g.cpu().numpy(), gref.numpy(), rtol=1e-4, atol=1e-5)


def test_adam_step_matches_optax_chain():
    from dips_gb300 import ops
    from dips_gb300.nn import n_params

    case = _parity.build_case("sphere", n=16, arch=(2, 16, 2, 16))
    P = n_params(case.gpu_arch())
    rng = np.random.default_rng(1)
    ref = O.ChainedAdam(P, lr=1e-3, decay_rate=0.9)
    opt = ops.AdamState(P, lr=1e-3, decay_rate=0.9)
    p_ref = case.params.copy()
    p_gpu = torch.as_tensor(case.params.copy(), device="cuda")
    for it in range(6):
        scale = 0.3 if it % 2 == 0 else 5.0  # below and above the clipping norm
        g = (rng.standard_normal(P) * scale / np.sqrt(P)).astype(F32)
        p_ref = ref.update(p_ref, g)
        opt.step(case.gpu_arch(), p_gpu, torch.as_tensor(g, device="cuda"))
    np.testing.assert_allclose(p_gpu.cpu().numpy(), p_ref, rtol=1e-5, atol=1e-7)
    assert int(opt.count.item()) == 6


@pytest.mark.parametrize("variant", ["polynomial", "rmsprop"])
def test_optimizer_variants_match_optax(variant):
    """get_optimizer's other options (solvers/optimizers.py:13-97): the chained Adam with the
    polynomial schedule (rate to 0 over transition_steps, here 3 of the 6 steps) and optax.rmsprop,
    through dips_adam_step and through the fused training step's tail."""
    from dips_gb300 import ops
    from dips_gb300.nn import n_params

    case = _parity.build_case("sphere", n=16, arch=(2, 16, 2, 16))
    P = n_params(case.gpu_arch())
    rng = np.random.default_rng(2)
    if variant == "polynomial":
        ref = O.ChainedAdam(P, lr=1e-3, transition_steps=3, schedule="polynomial")
        opt = ops.AdamState(P, lr=1e-3, transition_steps=3, schedule="polynomial")
    else:
        ref = O.RMSprop(P, lr=1e-3)
        opt = ops.AdamState(P, lr=1e-3, decay_rate=1.0, max_norm=float("inf"), b2=0.9, eps=1e-8, kind="rmsprop")
    p_ref = case.params.copy()
    p_gpu = torch.as_tensor(case.params.copy(), device="cuda")
    for it in range(6):
        scale = 0.3 if it % 2 == 0 else 5.0
        g = (rng.standard_normal(P) * scale / np.sqrt(P)).astype(F32)
        p_ref = ref.update(p_ref, g)
        opt.step(case.gpu_arch(), p_gpu, torch.as_tensor(g, device="cuda"))
    np.testing.assert_allclose(p_gpu.cpu().numpy(), p_ref, rtol=1e-5, atol=1e-7)
    if variant == "polynomial":  # the last three steps had rate 0
        assert float(ref.step_size()) == 0.0


@pytest.mark.parametrize("variant", ["polynomial", "rmsprop"])
def test_train_steps_with_optimizer_variants_track_oracle(variant):
    from dips_gb300 import ops

    case = _parity.build_case("sphere", n=16, arch=(1, 1, 2, 10))
    lvl = case.gpu_level()
    arch = case.gpu_arch()
    P = case.params.size
    params = torch.as_tensor(case.params.copy(), device="cuda")
    if variant == "polynomial":
        opt = ops.AdamState(P, lr=1e-3, transition_steps=4, schedule="polynomial")
        ref = O.ChainedAdam(P, lr=1e-3, transition_steps=4, schedule="polynomial")
    else:
        opt = ops.AdamState(P, lr=1e-3, decay_rate=1.0, max_norm=float("inf"), b2=0.9, eps=1e-8, kind="rmsprop")
        ref = O.RMSprop(P, lr=1e-3)
    ws = ops.StepWorkspace(arch, lvl.n, lvl.max_jobs(lvl.n))
    loss = torch.empty((), dtype=torch.float64, device="cuda")
    p_ref = case.params.copy()
    rg = case.oracle_geometry()
    for _ in range(5):
        ops.train_step(arch, params, opt, lvl, None, ws, loss)
        l_ref, g_ref = L.loss_and_grad(p_ref, case.arch, rg)
        p_ref = ref.update(p_ref, g_ref)
        torch.cuda.synchronize()
        assert abs(float(loss) - l_ref) <= 1e-4 * abs(l_ref)
    np.testing.assert_allclose(params.cpu().numpy(), p_ref, rtol=1e-4, atol=1e-6)


def test_train_steps_track_oracle():
    from dips_gb300 import ops

    case = _parity.build_case("sphere", n=16, arch=(1, 1, 2, 10))
    lvl = case.gpu_level()
    arch = case.gpu_arch()
    P = case.params.size
    params = torch.as_tensor(case.params.copy(), device="cuda")
    opt = ops.AdamState(P, lr=1e-3, decay_rate=0.9)
    ws = ops.StepWorkspace(arch, lvl.n, lvl.max_jobs(lvl.n))
    loss = torch.empty((), dtype=torch.float64, device="cuda")
    ref = O.ChainedAdam(P, lr=1e-3, decay_rate=0.9)
    p_ref = case.params.copy()
    rg = case.oracle_geometry()
    for _ in range(5):
        ops.train_step(arch, params, opt, lvl, None, ws, loss)
        l_ref, g_ref = L.loss_and_grad(p_ref, case.arch, rg)
        p_ref = ref.update(p_ref, g_ref)
        torch.cuda.synchronize()
        assert abs(float(loss) - l_ref) <= 1e-4 * abs(l_ref)
    np.testing.assert_allclose(params.cpu().numpy(), p_ref, rtol=1e-4, atol=1e-6)


def test_batch_ids_are_a_permutation():
    from dips_gb300 import ops

    n, B = 10007, 1000
    seen = np.concatenate([ops.batch_ids(n, B, epoch=3, batch_index=b, seed=7).cpu().numpy() for b in range(10)])
    assert len(np.unique(seen)) == seen.size and seen.min() >= 0 and seen.max() < n
    other = ops.batch_ids(n, B, epoch=4, batch_index=0, seed=7).cpu().numpy()
    assert not np.array_equal(other, seen[:B])


def test_autotune_choice_and_unchanged_results():
    from dips_gb300 import ops

    case = _parity.build_case("sphere", n=20, arch=(3, 32, 3, 32), level=0)
    lg0, gg0 = case.gpu_loss_grad()
    lvl = case.gpu_level()
    a = case.gpu_arch()
    params = torch.as_tensor(case.params, device="cuda")
    ws = ops.StepWorkspace(a, lvl.n, lvl.max_jobs(lvl.n), "cuda")
    nw = ops.autotune(a, params, lvl, None, ws)
    assert nw in (8, 10, 12)
    lg1, gg1 = case.gpu_loss_grad()
    assert abs(lg1 - lg0) <= 1e-6 * abs(lg0)
    np.testing.assert_allclose(gg1, gg0, rtol=1e-4, atol=1e-6 * np.max(np.abs(gg0)))
    # shapes without a tunable kernel report 0
    small = _parity.build_case("sphere", n=12, arch=(1, 1, 2, 10), level=0)
    slvl = small.gpu_level()
    sa = small.gpu_arch()
    sws = ops.StepWorkspace(sa, slvl.n, slvl.max_jobs(slvl.n), "cuda")
    assert ops.autotune(sa, torch.as_tensor(small.params, device="cuda"), slvl, None, sws) == 0


@pytest.mark.parametrize("arch", [(3, 32, 3, 32), (2, 16, 2, 16)])
def test_packed_bulk_records_give_the_gathered_result(arch):
    """The bulk records packed once per level (dips_pack_bulk_records) and the per-step gather
    from the record arrays give bit-identical residuals and the same loss."""
    from dips_gb300 import ops

    case = _parity.build_case("star", n=20, arch=arch, level=1, batch=3000)
    lvl = case.gpu_level()
    a = case.gpu_arch()
    params = torch.as_tensor(case.params, device="cuda")
    ids = case.gpu_batch_ids()
    l0, r0, _ = ops.residual_forward(a, params, lvl, ids, want_residual=True)
    packed = lvl.desc.bulk_rec
    assert packed
    try:
        lvl.desc.bulk_rec = None
        l1, r1, _ = ops.residual_forward(a, params, lvl, ids, want_residual=True)
    finally:
        lvl.desc.bulk_rec = packed
    assert torch.equal(r0, r1)
    assert abs(float(l0) - float(l1)) <= 1e-12 * abs(float(l0))


@pytest.mark.parametrize(
    "name,n,arch,level,batch",
    [
        ("sphere", 16, (1, 1, 2, 10, 2, 16, 1.0), 0, None),
        ("star", 16, (3, 32, 3, 32, 1, 32, 1.0), 1, None),
        ("star", 20, (2, 16, 2, 16, 3, 8, 2.0), 0, 2000),
    ],
)
def test_learned_preconditioner_loss_and_gradient(name, n, arch, level, batch):
    """P(coeffs) = 0.5 + s sigmoid(MLP(coeffs)) multiplies each residual (discretization.py:339,
    :419-420); its parameters follow the networks' in the flat vector and get their gradient too."""
    case = _parity.build_case(name, n=n, arch=arch, level=level, batch=batch, batch_seed=3)
    lg, gg = case.gpu_loss_grad()
    lr, gr = case.oracle_loss_grad()
    assert abs(lg - lr) <= LOSS_RTOL * abs(lr), (lg, lr)
    _grad_close(gg, gr)
    from dips_gb300 import nn

    a = case.gpu_arch()
    npre = nn.n_params(a) - nn.n_params(nn.Arch(a.m_layers, a.m_width, a.p_layers, a.p_width))
    assert npre > 0
    gp, rp = np.asarray(gg)[-npre:], np.asarray(gr)[-npre:]
    assert np.linalg.norm(gp - rp) <= GRAD_RTOL * np.linalg.norm(rp)


def test_quadratic_interpolation_bit_exact():
    from dips_gb300 import levelset, mesh

    g = mesh.uniform_grid(23)
    rng = np.random.default_rng(9)
    vals = rng.standard_normal(23 ** 3).astype(F32)
    T = O.Trilinear(vals, g.x, g.y, g.z)
    ls = levelset.LevelSetGrid(g, vals)
    pts = rng.uniform(-1.3, 1.3, (20000, 3)).astype(F32)  # inside, near and beyond the box
    got = ls.quadratic(torch.as_tensor(pts, device="cuda")).cpu().numpy()
    np.testing.assert_array_equal(got, T.quadratic(pts))
