"""The CPU oracle pinned against the reference's own known answers and against
mathematics it must satisfy (no GPU).

Pins: the reference's geometric-integration test (tests/test_geometric_integrations.py:
172-182: sum of interface areas of the r=0.5 sphere = pi +- 0.02 and enclosed volume =
pi/6 +- 0.02 on 128^3 over [-2,2]^3), central finite differences of the loss, jax's
pinv cutoff, linear exactness of the trilinear interpolant, and optax's Adam chain.
Residual/loss/gradient values are "parity unpinned": the reference's tests hold none.
"""

import numpy as np
import pytest
import torch

import _parity

O = _parity.O
L = _parity.L
F32 = np.float32


def test_geometry_known_answer_sphere_area_and_volume():
    x = O.linspace_f32(-2, 2, 128)
    P = O.grid_points(x, x, x)
    phi = O.perturb(np.sqrt((P * P).sum(1, dtype=F32)) - F32(0.5))
    T = O.Trilinear(phi, x, x, x)
    h = np.array([O.grid_spacing(x)] * 3, F32)
    # cells farther than 1.5 h from the interface are not crossed: area 0, volume h^3 or 0
    near = np.abs(phi) <= 1.5 * h[0]
    inside_far = (phi < -1.5 * h[0]).sum()
    geo = O.CellGeometry(T, P[near], h)
    one = lambda q: np.ones(q.shape[0], F32)  # noqa: E731
    area = O.interface_integral(geo, one).astype(np.float64).sum()
    vol = O.negative_volume_integral(geo, one).astype(np.float64).sum() + inside_far * float(h[0]) ** 3
    assert abs(area - np.pi) < 0.02
    assert abs(vol - 4.0 * np.pi * 0.5**3 / 3.0) < 0.02
    # the far cells really are uncrossed with the full (or empty) volume
    far = np.nonzero(~near)[0][:: max(1, (~near).sum() // 2000)]
    gf = O.CellGeometry(T, P[far], h)
    assert np.all(gf.crossed != 0)
    vf = O.negative_volume_integral(gf, one)
    np.testing.assert_allclose(vf, np.where(phi[far] < 0, h[0] ** 3, 0.0), rtol=1e-5, atol=1e-12)


def test_trilinear_is_exact_on_linear_fields_with_the_first_cell_quirk():
    x = O.linspace_f32(-1, 1, 9)
    P = O.grid_points(x, x, x)
    vals = (0.3 * P[:, 0] - 0.7 * P[:, 1] + 0.2 * P[:, 2] + 0.1).astype(F32)
    T = O.Trilinear(vals, x, x, x)
    rng = np.random.default_rng(0)
    q = rng.uniform(-1, 1, (2000, 3)).astype(F32)
    ref = 0.3 * q[:, 0] - 0.7 * q[:, 1] + 0.2 * q[:, 2] + 0.1
    np.testing.assert_allclose(T(q), ref, atol=2e-6)
    # the lower-left index is clamped to 2: a point in the first real cell uses cell [2,3]
    assert T._index(np.array([x[0] + 0.1 * (x[1] - x[0])], F32), T.xx)[0] == 2


def test_pinv_restatement_matches_numpy_pinv():
    X = O.xijk(np.array([0.1, 0.1, 0.1], F32))
    rng = np.random.default_rng(2)
    w = (rng.uniform(size=(200, 27)) < 0.4).astype(F32)
    w[0] = 0
    w[1, :] = 0
    w[1, [4, 22]] = 1  # rank 1: collinear points
    D = O.pinv_lsq(X, w)
    X64 = X.astype(np.float64)
    for i in range(w.shape[0]):
        W = np.diag(w[i].astype(np.float64))
        ref = np.linalg.pinv(X64.T @ W @ X64, rcond=10 * 3 * np.finfo(np.float32).eps) @ (W @ X64).T
        np.testing.assert_allclose(D[i], ref, rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("name,arch,level", [("sphere", (1, 1, 2, 10), 0), ("star", (2, 8, 2, 8), 1)])
def test_oracle_gradient_matches_central_differences(name, arch, level):
    case = _parity.build_case(name, n=12, arch=arch, level=level)
    rg = case.oracle_geometry()
    w = case.params.astype(np.float64)
    _, g = L.loss_and_grad(w, case.arch, rg, torch.float64)
    rng = np.random.default_rng(4)
    for i in rng.choice(w.size, min(16, w.size), replace=False):
        e = 1e-3
        wp, wm = w.copy(), w.copy()
        wp[i] += e
        wm[i] -= e
        lp = float(L.loss(torch.tensor(wp), case.arch, rg, torch.float64))
        lm = float(L.loss(torch.tensor(wm), case.arch, rg, torch.float64))
        fd = (lp - lm) / (2 * e)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i])) + 1e-4 * np.abs(g).max()


def test_fp32_oracle_error_against_fp64():
    case = _parity.build_case("sphere", n=16, arch=(1, 1, 2, 10))
    l32, g32 = case.oracle_loss_grad(torch.float32)
    l64, g64 = case.oracle_loss_grad(torch.float64)
    assert abs(l32 - l64) / abs(l64) < 1e-6
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) < 1e-5


def test_adam_chain_semantics():
    opt = O.ChainedAdam(3, lr=1e-2, decay_rate=0.5, transition_steps=2)
    p = np.zeros(3, F32)
    g = np.array([3.0, 4.0, 0.0], F32)  # norm 5 -> clipped to 1
    p1 = opt.update(p, g)
    # first Adam step moves each nonzero coordinate by -lr * sign(g) (bias-corrected)
    np.testing.assert_allclose(p1, [-1e-2, -1e-2, 0.0], rtol=1e-5, atol=1e-8)
    p2 = opt.update(p1, g)
    # second step: lr * 0.5^(1/2) schedule at count 1
    np.testing.assert_allclose(p2 - p1, [-1e-2 * 0.5**0.5] * 2 + [0.0], rtol=1e-4, atol=1e-8)


def test_h_schedule_and_sequential_batches():
    assert [O.h_level(200, e) for e in (0, 49, 50, 149, 150, 199)] == [0, 0, 1, 2, 3, 3]
    assert O.sequential_batches(32768, 262144) == (1, 32768, 0)
    assert O.sequential_batches(1000, 300) == (4, 300, 200)


def test_quadratic_interpolation_reproduces_a_convex_quadratic():
    """The non-oscillatory quadratic interpolant (interpolate.py:572-759) subtracts
    0.5 t (1 - t) min|D2| per axis from the trilinear value; for x^2 + y^2 + z^2 (second
    differences 2 dx^2 everywhere) that cancels the trilinear error exactly."""
    from dips_gb300 import mesh

    g = mesh.uniform_grid(17)
    X, Y, Z = np.meshgrid(g.x, g.y, g.z, indexing="ij")
    vals = (X * X + Y * Y + Z * Z).astype(np.float32)
    T = O.Trilinear(vals.reshape(-1), g.x, g.y, g.z)
    rng = np.random.default_rng(2)
    p = rng.uniform(-0.8, 0.8, (4000, 3)).astype(np.float32)
    exact = (p ** 2).sum(1)
    q = T.quadratic(p)
    t = T(p)
    assert np.max(np.abs(q - exact)) < 2e-5
    assert np.max(np.abs(t - exact)) > 100 * np.max(np.abs(q - exact))


def test_polynomial_schedule_and_rmsprop_semantics():
    # polynomial_schedule(lr, end 0, power 1, transition_steps 4): lr (1 - min(count, 4) / 4)
    opt = O.ChainedAdam(1, lr=1e-2, transition_steps=4, schedule="polynomial")
    steps = []
    for _ in range(6):
        steps.append(float(opt.step_size()))
        opt.update(np.zeros(1, F32), np.ones(1, F32))
    np.testing.assert_allclose(steps, [1e-2, 7.5e-3, 5e-3, 2.5e-3, 0.0, 0.0], rtol=1e-6, atol=1e-12)
    # rmsprop: first step -lr g / sqrt((1 - decay) g^2 + eps)
    r = O.RMSprop(2, lr=1e-2)
    p1 = r.update(np.zeros(2, F32), np.array([2.0, -0.5], F32))
    np.testing.assert_allclose(p1, [-1e-2 * 2 / np.sqrt(0.1 * 4), 1e-2 * 0.5 / np.sqrt(0.1 * 0.25)], rtol=1e-5)
