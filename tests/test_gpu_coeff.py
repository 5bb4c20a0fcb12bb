"""The gradient of the total loss with respect to a physical coefficient, the networks fixed: the
records' exact tangent (dips_geometry_assemble_tangent) pushed through the residual
(dips_loss_coeff_tangent), against central finite differences of the loss with the records
re-assembled at the perturbed coefficient (Richardson-extrapolated, so the FD error is O(eps^4)).

The headline case is d loss / d mu+ of the irregular-blob problem (mu- = 1, mu+ = 100, MLP 4x64 on
the TF32 tensor-core engine); the FD and the tangent see the same network values, so TF32 rounding
cancels out of the comparison.
"""

import numpy as np
import pytest
import torch

import _parity
from dips_gb300 import levelset, mesh, nn, ops, problems
from dips_gb300.records import FVLevel

pytestmark = pytest.mark.gpu
F32 = np.float32


def _setup(name, n, arch, seed=3):
    pr = problems.blob_problem() if name == "blob" else _parity.make_problem(name)
    g = mesh.uniform_grid(n)
    ls = levelset.LevelSetGrid.from_callable(g, lambda r: levelset.perturb(pr["phi"](r)))
    pts = torch.as_tensor(g.R, device="cuda")
    h = np.array([g.dx, g.dy, g.dz], F32)
    a = nn.Arch(*arch)
    params = torch.as_tensor(nn.init_params(a, seed), device="cuda")
    return pr, ls, pts, h, a, params


def _fns(pr, **over):
    keys = ("mu_m", "mu_p", "k_m", "k_p", "f_m", "f_p", "g", "alpha", "beta")
    f = {k: pr[k] for k in keys}
    f.update(over)
    return f


def _loss(a, params, ls, pts, h, fns):
    lvl = FVLevel(ls, fns, pts, h)
    loss, _, _ = ops.residual_forward(a, params, lvl)
    return float(loss)


def _fd(a, params, ls, pts, h, pr, name, base, eps):
    def at(v):
        return _loss(a, params, ls, pts, h, _fns(pr, **{name: (lambda r, v=v: v)}))

    d1 = (at(base + eps) - at(base - eps)) / (2 * eps)
    d2 = (at(base + eps / 2) - at(base - eps / 2)) / eps
    return (4 * d2 - d1) / 3, d1


@pytest.mark.parametrize(
    "name,n,arch,mu_p",
    [("blob", 24, (4, 64, 4, 64), 100.0), ("sphere", 16, (3, 32, 3, 32), 10.0), ("sphere", 14, (1, 1, 2, 10), 10.0)],
)
def test_loss_gradient_wrt_mu_plus_matches_finite_differences(name, n, arch, mu_p):
    pr, ls, pts, h, a, params = _setup(name, n, arch)
    fns = _fns(pr, mu_p=lambda r: mu_p)
    lvl = FVLevel(ls, fns, pts, h, keep_geometry=True)
    t = lvl.coefficient_tangent({"mu_p": lambda r: 1.0})
    d = float(ops.loss_coefficient_derivative(a, params, lvl, t))
    fd, fd1 = _fd(a, params, ls, pts, h, pr, "mu_p", mu_p, 0.02 * mu_p)
    print(f"{name} {arch}: d loss / d mu+ = {d:.6e}, FD {fd:.6e} (plain central {fd1:.6e})")
    assert np.isfinite(d) and d != 0.0
    assert abs(d - fd) <= 2e-3 * abs(fd), (d, fd)


def test_linear_coefficients_tangent_against_finite_differences():
    """Two more directions: a constant k+ (diag and the centre coefficients) and a scaling of beta
    (the interface integral and the extrapolation's jump term), beta_s = (1 + s) beta."""
    pr, ls, pts, h, a, params = _setup("sphere", 14, (3, 32, 3, 32))
    lvl = FVLevel(ls, _fns(pr, k_p=lambda r: 0.7), pts, h, keep_geometry=True)
    d = float(ops.loss_coefficient_derivative(a, params, lvl, lvl.coefficient_tangent({"k_p": lambda r: 1.0})))
    # k V u is small beside the fluxes at this h, so the step is large (the loss is smooth in k)
    fd, _ = _fd(a, params, ls, pts, h, pr, "k_p", 0.7, 0.5)
    assert abs(d - fd) <= 2e-3 * abs(fd), ("k_p", d, fd)

    beta = pr["beta"]
    lvl = FVLevel(ls, _fns(pr), pts, h, keep_geometry=True)
    d = float(ops.loss_coefficient_derivative(a, params, lvl, lvl.coefficient_tangent({"beta": beta})))

    def at(s):
        return _loss(a, params, ls, pts, h, _fns(pr, beta=lambda r, s=s: (1.0 + s) * beta(r)))

    e = 0.02
    fd = (4 * (at(e / 2) - at(-e / 2)) / e - (at(e) - at(-e)) / (2 * e)) / 3
    assert abs(d - fd) <= 2e-3 * abs(fd), ("beta", d, fd)


def test_tangent_records_match_their_finite_differences():
    """The record tangents themselves (d diag, d lhs0, d rod, d A) against central differences of
    the assembled records at mu+ -+ eps (FP32 records: compared where the change is resolved)."""
    pr, ls, pts, h, a, params = _setup("sphere", 14, (3, 32, 3, 32))
    mu, eps = 10.0, 0.05
    lvl = FVLevel(ls, _fns(pr, mu_p=lambda r: mu), pts, h, keep_geometry=True)
    t = lvl.coefficient_tangent({"mu_p": lambda r: 1.0})
    lp = FVLevel(ls, _fns(pr, mu_p=lambda r: mu + eps), pts, h)
    lm = FVLevel(ls, _fns(pr, mu_p=lambda r: mu - eps), pts, h)
    # the written job slots: a point's first cnt_m and last cnt - cnt_m of its capacity
    off, cnt, cm = (x.cpu().numpy().astype(np.int64) for x in (lvl.job_off, lvl.cnt, lvl.cnt_m))
    idx = np.arange(off[-1])
    pt = np.searchsorted(off, idx, side="right") - 1
    local, cap = idx - off[pt], off[pt + 1] - off[pt]
    used = torch.as_tensor((local < cm[pt]) | (local >= cap - (cnt[pt] - cm[pt])), device="cuda")
    for other in (lp, lm):  # the same jobs: no branch of the assembly flips between mu+ -+ eps
        assert torch.equal(other.cnt, lvl.cnt) and torch.equal(other.cnt_m, lvl.cnt_m)
        assert torch.equal(other.job_code[: off[-1]][used], lvl.job_code[: off[-1]][used])
    for f in ("diag", "lhs0", "rod", "job_A"):
        pick = (lambda x: x[: off[-1]][used]) if f == "job_A" else (lambda x: x)
        fd = ((pick(getattr(lp, f)).double() - pick(getattr(lm, f)).double()) / (2 * eps)).cpu().numpy()
        tg = pick(getattr(t, f)).double().cpu().numpy()
        scale = np.abs(fd).max()
        assert scale > 0 or f == "lhs0"
        np.testing.assert_allclose(tg, fd, atol=2e-3 * max(scale, 1e-12), rtol=2e-3, err_msg=f)


def test_preconditioned_arch_is_refused():
    pr, ls, pts, h, _, _ = _setup("sphere", 12, (1, 1, 2, 10))
    a = nn.Arch(1, 1, 2, 10, 1, 8, 1.0)
    params = torch.as_tensor(nn.init_params(a, 1), device="cuda")
    lvl = FVLevel(ls, _fns(pr), pts, h, keep_geometry=True)
    t = lvl.coefficient_tangent({"mu_p": lambda r: 1.0})
    with pytest.raises(RuntimeError):
        ops.loss_coefficient_derivative(a, params, lvl, t)
