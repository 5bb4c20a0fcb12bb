"""Plain method on the GPU: the FV operator of a nodal vector against the oracle, and
BiCGSTAB against a float64 direct solve of the oracle's operator."""

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

L = _parity.L


def _nodal_lookup(n, h0):
    """Network values replaced by grid-node values of u (exact at nodes, as the reference's
    quadratic interpolant of a nodal vector is)."""

    def make(u):
        def values(net, x, phi_x):
            q = x.reshape(-1, 3).double()
            idx = torch.round((q + 1.0) / float(h0)).long().clamp(0, n - 1)
            lin = (idx[:, 0] * n + idx[:, 1]) * n + idx[:, 2]
            return u.to(q.dtype)[lin].reshape(x.shape[:-1])

        return values

    return make


def test_fv_residual_matches_oracle_nodal_operator():
    from dips_gb300 import krylov

    n = 20
    case = _parity.build_case("star", n=n)
    lvl = case.gpu_level()
    rng = np.random.default_rng(0)
    u = rng.standard_normal(n**3).astype(np.float32)
    got = krylov.fv_residual(lvl, (n, n, n), torch.as_tensor(u, device="cuda")).cpu().numpy()
    orig = L.nn_eval
    try:
        L.nn_eval = _nodal_lookup(n, case.grid.dx)(torch.as_tensor(u))
        ref = L.residual(torch.zeros(L.n_params(case.arch)), case.arch, case.oracle_geometry(), torch.float64).numpy()
    finally:
        L.nn_eval = orig
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-5 * np.abs(ref).max())


def test_bicgstab_solves_the_fv_system():
    import scipy.sparse.linalg as spla

    from dips_gb300 import krylov, problems

    n = 16
    case = _parity.build_case("sphere", n=n)
    lvl = case.gpu_level()
    ex = problems.exact_solution(case.fns, case.grid.R)
    res = krylov.bicgstab(lvl, (n, n, n), u_exact=torch.as_tensor(ex, device="cuda"), max_iter=2000, rtol=1e-6,
                          check_every=5)
    assert not res.breakdown and res.rel_residual <= 1e-6
    x = res.x.cpu().numpy().astype(np.float64)
    # float64 reference solve of the oracle's nodal operator
    rg = case.oracle_geometry()
    U = {}
    look = _nodal_lookup(n, case.grid.dx)
    orig = L.nn_eval
    try:
        z = torch.zeros(L.n_params(case.arch), dtype=torch.float64)
        L.nn_eval = lambda net, xx, ph: look(U["u"])(net, xx, ph)  # noqa: E731
        U["u"] = torch.zeros(n**3, dtype=torch.float64)
        r0 = L.residual(z, case.arch, rg, torch.float64).numpy()

        def mv(v):
            U["u"] = torch.as_tensor(v)
            return L.residual(z, case.arch, rg, torch.float64).numpy() - r0

        A = spla.LinearOperator((n**3, n**3), matvec=mv, dtype=np.float64)
        sol, info = spla.bicgstab(A, -r0, rtol=1e-10, maxiter=2000)
    finally:
        L.nn_eval = orig
    assert info == 0
    assert np.abs(x - sol).max() <= 1e-4 * np.abs(sol).max()
    err = np.abs(sol - ex).max() / np.abs(ex).max()
    assert abs(res.rel_linf - err) <= 1e-3


@pytest.mark.parametrize("key", _parity.reference_fixtures("fvop"))
def test_fv_residual_against_the_references_residual_vector(key):
    """dips_fv_residual against the reference's own residual_vector (trainer.py:883-890, via
    tests/golden/make_reference_golden.py) for a random nodal vector and the exact solution.

    The reference reads u through its non-oscillatory quadratic interpolant
    (interpolate.py:572-759).  At a node that is the nodal value, except in the first cell of an
    axis: its lower-left index is clamped to the second cell, so a node of the lowest layer gets
    2 u_1 - u_2 + min|second difference| -- not linear in u.  The library's operator reads the
    nodal values everywhere (a linear operator, which BiCGSTAB needs).  So rows whose stencil or
    regression cube reaches a node of the lowest layer of some axis -- the rows of the two lowest
    layers -- may differ; every other row must agree."""
    from golden import make_reference_golden as M

    from dips_gb300 import krylov

    fx = _parity.load_reference_fixture(key)
    prob = str(fx["problem"])
    n = int(fx["n"])
    case = _parity.Case(prob, n, (1, 1, 2, 10), 0, fns=M.problem(prob), phi=fx["phi"])
    lvl = case.gpu_level()
    rows = fx["rows"].astype(np.int64)
    ijk = np.stack(np.unravel_index(rows, (n, n, n)), 1)
    low = (ijk <= 1).any(1)
    assert low.sum() >= 64 and (~low).sum() >= 64
    for ukey, rkey in (("u_rand", "res_rand"), ("u_exact", "res_exact")):
        got = krylov.fv_residual(lvl, (n, n, n), torch.as_tensor(fx[ukey], device="cuda")).cpu().numpy()[rows]
        ref = fx[rkey]
        scale = float(np.max(np.abs(ref)))
        err = np.abs(got - ref)
        assert float(err[~low].max()) <= 3e-5 * scale, (ukey, float(err[~low].max()), scale)
        bad = err > 3e-5 * scale
        assert not (bad & ~low).any()


def test_bicgstab_without_packed_records_and_on_a_larger_grid():
    """Every row through the general-row path (no packed bulk records: the bulk rows become light
    rows of 7 jobs) gives the solution of the packed solve, on a 40^3 grid whose general rows fill
    several job-count bins."""
    from dips_gb300 import krylov, problems

    n = 40
    case = _parity.build_case("sphere", n=n)
    lvl = case.gpu_level()
    ex = torch.as_tensor(problems.exact_solution(case.fns, case.grid.R), device="cuda")
    a = krylov.bicgstab(lvl, (n, n, n), u_exact=ex, max_iter=3000, rtol=1e-6, check_every=10)
    saved = lvl.desc.bulk_rec
    try:
        lvl.desc.bulk_rec = None
        b = krylov.bicgstab(lvl, (n, n, n), u_exact=ex, max_iter=3000, rtol=1e-6, check_every=10)
    finally:
        lvl.desc.bulk_rec = saved
    for r in (a, b):
        assert not r.breakdown and r.rel_residual <= 1e-6
    xa, xb = a.x.cpu().numpy(), b.x.cpu().numpy()
    assert np.abs(xa - xb).max() <= 1e-4 * np.abs(xa).max()
    assert abs(a.rel_linf - b.rel_linf) <= 1e-3
