"""The oracle against golden vectors computed by the reference's own code (no GPU).

The fixtures ``tests/golden/ref_*.npz`` were written by ``tests/golden/make_reference_golden.py``,
which runs the reference's unmodified discretization, geometry, level-set and interpolation
modules on a numpy stand-in for jax.  Each holds, for a seeded batch of grid points at one
stencil level: the 26 cell values, the interface integral and the crossing flag per point,
[lhs/diag, rhs/diag] per point, the loss with x64 off and on, and three directional derivatives
of the x64 loss (fourth-order central differences).  Here the oracle, given the same phi samples,
parameters and batch, must reproduce them:

* crossing flags exactly;
* cell values and interface integrals to float32 rounding (rtol 1e-5);
* residuals to 3e-5 of the residual scale (float32 sums of the 64-wide layers are ordered
  differently), the float32 loss to 1e-5 relative (the parity bar);
* the float64 loss to 1e-6 relative (the reference's x64 run keeps its explicit float32 casts of
  points and geometry; the oracle keeps its geometry in float32);
* the gradient along each direction to 1e-4 of the gradient's norm (the parity bar).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import _parity  # noqa: E402

KEYS = _parity.reference_fixtures()


def test_reference_fixtures_present():
    assert len(KEYS) >= 8, KEYS
    assert len(_parity.reference_fixtures("fvop")) >= 2


@pytest.fixture(scope="module")
def cases():
    return {}


def _case(cases, key):
    if key not in cases:
        case, fx = _parity.reference_case(key)
        rg = case.oracle_geometry()
        cases[key] = (case, fx, rg)
    return cases[key]


@pytest.mark.parametrize("key", KEYS)
def test_oracle_geometry_matches_reference(cases, key):
    case, fx, rg = _case(cases, key)
    np.testing.assert_array_equal(np.asarray(rg.crossed_p, np.float32), fx["crossed"])
    c = np.asarray(rg.coeffs, np.float32)
    scale = float(np.max(np.abs(fx["coeff26"])))
    np.testing.assert_allclose(c, fx["coeff26"], rtol=1e-5, atol=1e-6 * scale)
    b = np.asarray(rg.beta_int, np.float32)
    ref_b = fx["beta_int"]
    fin = np.isfinite(ref_b)
    # a NaN interface integral (beta NaN at the zero-padding triangles) is NaN in both
    np.testing.assert_array_equal(np.isfinite(b), fin)
    bs = float(np.max(np.abs(ref_b[fin]))) if fin.any() else 1.0
    np.testing.assert_allclose(b[fin], ref_b[fin], rtol=1e-5, atol=1e-6 * bs)


@pytest.mark.parametrize("key", KEYS)
def test_oracle_residual_and_loss_match_reference(cases, key):
    case, fx, rg = _case(cases, key)
    res = case.oracle_residual(torch.float32)
    ref = fx["lhs_rhs"][:, 0] - fx["lhs_rhs"][:, 1]
    scale = float(np.max(np.abs(ref)))
    assert float(np.max(np.abs(res - ref))) <= 3e-5 * scale
    l32, _ = case.oracle_loss_grad(torch.float32)
    assert abs(float(l32) - float(fx["loss32"])) <= 1e-5 * abs(float(fx["loss32"]))
    l64, _ = case.oracle_loss_grad(torch.float64)
    assert abs(float(l64) - float(fx["loss64"])) <= 1e-6 * abs(float(fx["loss64"]))


@pytest.mark.parametrize("key", KEYS)
def test_oracle_gradient_matches_reference_directional_derivatives(cases, key):
    case, fx, rg = _case(cases, key)
    _, g64 = case.oracle_loss_grad(torch.float64)
    g64 = np.asarray(g64, np.float64)
    d = fx["dirs"].astype(np.float64) @ g64
    gn = float(np.linalg.norm(g64))
    np.testing.assert_allclose(d, fx["dloss64"], rtol=0, atol=1e-4 * gn)


FV_KEYS = _parity.reference_fixtures("fvop")


def _quadratic_lookup(phi_case, u):
    """Network values replaced by the reference's non-oscillatory quadratic interpolant of the
    nodal vector u (interpolate.py:572-759), as compute_Ax_and_b_discrete_fn reads u."""
    g = phi_case.grid
    T = _parity.O.Trilinear(u, g.x, g.y, g.z)

    def values(net, x, phi_x):
        q = x.detach().reshape(-1, 3).numpy().astype(np.float32)
        return torch.as_tensor(T.quadratic(q)).to(x.dtype).reshape(x.shape[:-1])

    return values


@pytest.mark.parametrize("key", FV_KEYS)
def test_oracle_discrete_operator_matches_reference(key):
    """The reference's own residual_vector (trainer.py:883-890) of a random nodal vector and of
    the exact solution against the oracle's residual with u read through the quadratic
    interpolant, on every fixture row (the first-cell rows included)."""
    from golden import make_reference_golden as M

    fx = _parity.load_reference_fixture(key)
    prob = str(fx["problem"])
    n = int(fx["n"])
    case = _parity.Case(prob, n, (1, 1, 2, 10), 0, fns=M.problem(prob), phi=fx["phi"], ids=fx["rows"])
    rg = case.oracle_geometry()
    L = _parity.L
    orig = L.nn_eval
    try:
        for ukey, rkey in (("u_rand", "res_rand"), ("u_exact", "res_exact")):
            L.nn_eval = _quadratic_lookup(case, fx[ukey])
            got = L.residual(torch.zeros(L.n_params(case.arch)), case.arch, rg, torch.float32).numpy()
            ref = fx[rkey]
            scale = float(np.max(np.abs(ref)))
            assert float(np.max(np.abs(got - ref))) <= 3e-5 * scale, (ukey, float(np.max(np.abs(got - ref))), scale)
    finally:
        L.nn_eval = orig
