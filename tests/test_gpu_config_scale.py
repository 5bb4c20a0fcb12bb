"""Parity at the benchmark configurations' own sizes, on 4,096-point samples.

Every other parity test runs on grids of 12^3 to 32^3.  Here the CUDA path builds its records
over the whole training grid of each benchmark configuration, the level set sampled on the
device, and the oracle recomputes the same 4,096 seeded points from the same level-set samples:

* configuration 2: the 128^3 sphere, 3x32 networks, at h = dx and h = dx/2;
* configuration 3: the 256^3 star (variable mu, k+ = 1), 3x32;
* configuration 4: one linearised Poisson-Boltzmann molecule at its own grid side (k+ = 0.1,
  Gaussian charges, zero Dirichlet data), 2x16, and a 3-instance persistent step whose losses
  and first Adam moments are checked against each instance's oracle loss and clipped gradient;
* configuration 5: the 500-Gaussian blob on a 256^3 level-set grid with a 192^3 training grid,
  4x64 on the TF32 tensor-core engine, against the FP64 oracle.

Bars: the FP32 engines as in the small-grid tests (loss 1e-5, gradient 1e-4 relative); the TF32
engine against FP64, loss 5e-5 (measured 1.1e-5 here: TF32 operands carry 10 mantissa bits and
mu+ = 100 scales the jump terms) and gradient 1e-3 relative.
"""

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

L = _parity.L
O = _parity.O
F32 = np.float32


def _params(arch, seed):
    p = L.init_params(arch, seed)
    rng = np.random.default_rng(seed + 1000)
    return (p + F32(0.02) * rng.standard_normal(p.shape).astype(F32)).astype(F32)


def _ids(n, batch, seed, phi=None, dx=None):
    """A seeded sample of the grid points; with phi, half of it within 2.5 dx of the interface
    (where the cube jobs and the extrapolation are), the rest uniform."""
    rng = np.random.default_rng(seed)
    if phi is None:
        return np.sort(rng.choice(n, batch, replace=False)).astype(np.int32)
    near = np.nonzero(np.abs(phi) < 2.5 * dx)[0]
    a = rng.choice(near, min(batch // 2, near.size), replace=False)
    rest = np.setdiff1d(np.arange(n), a)
    b = rng.choice(rest, batch - a.size, replace=False)
    return np.sort(np.concatenate([a, b])).astype(np.int32)


def _run(fns, n_tr, n_ls, arch, level=0, batch=4096, seed=0, keep_geometry=False):
    from dips_gb300 import levelset, mesh, nn, ops, records

    g_tr = mesh.uniform_grid(n_tr)
    g_ls = g_tr if n_ls == n_tr else mesh.uniform_grid(n_ls)
    ls = levelset.LevelSetGrid.from_callable(g_ls, lambda r: levelset.perturb(fns["phi"](r)))
    phi = ls.phi.cpu().numpy()
    h = np.array([g_tr.dx, g_tr.dy, g_tr.dz], F32) * F32(0.5**level)
    lvl = records.FVLevel(ls, fns, torch.as_tensor(g_tr.R, device="cuda"), h, keep_geometry=keep_geometry)
    phi_tr = ls(torch.as_tensor(g_tr.R, device="cuda")).cpu().numpy()
    ids = _ids(g_tr.R.shape[0], batch, seed, phi_tr, float(g_tr.dx))
    a = L.Arch(*arch)
    ga = nn.Arch(*arch)
    params = _params(a, seed)
    pt = torch.as_tensor(params, device="cuda")
    it = torch.as_tensor(ids, device="cuda")
    loss, res, ws = ops.residual_forward(ga, pt, lvl, it, want_residual=True)
    grad = ops.residual_backward(ga, pt, lvl, it, ws)
    torch.cuda.synchronize()
    flags = lvl.flags.cpu().numpy()[ids] if keep_geometry else None
    out = dict(loss=float(loss), res=res.cpu().numpy(), grad=grad.cpu().numpy().astype(np.float64), flags=flags)
    del lvl, ls, ws
    torch.cuda.empty_cache()
    rg = L.ResidualGeometry(L.Problem(phi, g_ls.x, g_ls.y, g_ls.z, fns), g_tr.R[ids], h)
    return out, rg, params, a


def _check_fp32(out, rg, params, a):
    l32, g32 = L.loss_and_grad(params, a, rg, torch.float32)
    assert abs(out["loss"] - float(l32)) <= 1e-5 * abs(float(l32)), (out["loss"], float(l32))
    g32 = np.asarray(g32, np.float64)
    err = np.linalg.norm(out["grad"] - g32) / np.linalg.norm(g32)
    assert err <= 1e-4, err
    r = L.residual(torch.tensor(params), a, rg, torch.float32).numpy()
    assert float(np.max(np.abs(out["res"] - r))) <= 1e-5 * float(np.max(np.abs(r)))
    if out["flags"] is not None:
        cp = ((out["flags"].astype(np.uint32) >> 1) & 3).astype(np.int64) - 1
        np.testing.assert_array_equal(cp, rg.crossed_p.astype(np.int64))


@pytest.mark.parametrize("level", [0, 1])
def test_config2_sphere_128_3x32(level):
    from dips_gb300 import problems

    out, rg, params, a = _run(problems.sphere_problem(), 128, 128, (3, 32, 3, 32), level=level, seed=level,
                              keep_geometry=True)
    assert int((rg.crossed_s == 0).any(axis=1).sum()) > 500  # the sample reaches the interface
    _check_fp32(out, rg, params, a)


def test_config3_star_256_3x32():
    from dips_gb300 import problems

    out, rg, params, a = _run(problems.star_problem(), 256, 256, (3, 32, 3, 32), seed=2)
    _check_fp32(out, rg, params, a)


def test_config4_lpbe_instance_2x16():
    from dips_gb300 import problems

    side, c, r, q = problems.lpbe_instances(64, seed=0)[0]
    out, rg, params, a = _run(problems.lpbe_problem(c, r, q), side, side, (2, 16, 2, 16), seed=3)
    _check_fp32(out, rg, params, a)


def test_config4_persistent_three_instances_against_oracle():
    """One persistent multi-instance step on given ids: each instance's loss against its oracle
    FP32 loss, and its first Adam moment (0.1 x the clipped gradient, optax clip_by_global_norm
    1.0 then scale_by_adam) against the oracle's clipped gradient."""
    from dips_gb300 import batch, nn, problems

    insts = [(side, problems.lpbe_problem(c, r, q)) for side, c, r, q in problems.lpbe_instances(64, seed=0)[:3]]
    arch = nn.Arch(2, 16, 2, 16)
    b = batch.InstanceBatch(insts, arch, batch=4096, lr=1e-3, seed=3, persistent=True)
    assert b.persistent
    p0 = [it.params.cpu().numpy().copy() for it in b.items]
    idss = []
    for k, it in enumerate(b.items):
        ids = _ids(it.level.n, it.batch, 20 + k)
        it.ids.copy_(torch.as_tensor(ids, device="cuda"))
        idss.append(ids)
    losses = b.step_with_ids().cpu().numpy()
    a = L.Arch(2, 16, 2, 16)
    for k, (it, (side, prob)) in enumerate(zip(b.items, insts)):
        g = it.grid
        rg = L.ResidualGeometry(L.Problem(it.ls.phi.cpu().numpy(), g.x, g.y, g.z, prob), g.R[idss[k]],
                                np.array([g.dx, g.dy, g.dz], F32))
        l32, g32 = L.loss_and_grad(p0[k], a, rg, torch.float32)
        assert abs(losses[k] - float(l32)) <= 1e-5 * abs(float(l32)), (k, losses[k], float(l32))
        g32 = np.asarray(g32, np.float64)
        gn = np.linalg.norm(g32)
        clipped = g32 if gn < 1.0 else g32 / gn
        mu = it.opt.mu.cpu().numpy().astype(np.float64) / 0.1
        err = np.linalg.norm(mu - clipped) / np.linalg.norm(clipped)
        assert err <= 1e-4, (k, err)


def test_config5_blob_256_level_set_192_training_4x64_tf32():
    from dips_gb300 import problems

    out, rg, params, a = _run(problems.blob_problem(), 192, 256, (4, 64, 4, 64), seed=4)
    l64, g64 = L.loss_and_grad(params, a, rg, torch.float64)
    # measured 1.1e-5 relative on a uniform sample of this problem (mu+ = 100)
    assert abs(out["loss"] - float(l64)) <= 5e-5 * abs(float(l64)), (out["loss"], float(l64))
    g64 = np.asarray(g64, np.float64)
    err = np.linalg.norm(out["grad"] - g64) / np.linalg.norm(g64)
    assert err <= 1e-3, err
