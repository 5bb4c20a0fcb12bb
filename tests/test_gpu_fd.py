"""The adjoint against central finite differences on 64 random parameters (h = 1e-3) for the
variable-coefficient star problem with the 3x32 networks (mu- = 1 + 0.5 sin xy,
mu+ = 20 + 5 cos z, k+ = 1; u- = exp(-|x|^2), u+ = cos(x+y+z)).

Two differences are taken: of the GPU's own FP32 loss (the adjoint must be the derivative of
what the kernels compute; FP32 rounding of the loss limits this to about a percent of the
largest component), and of the oracle's loss in FP64 (the adjoint must match the exact
derivative to FP32 accuracy).
"""

import numpy as np
import pytest
import torch

import _parity
from dips_gb300 import levelset, mesh, nn, ops, problems
from dips_gb300.records import FVLevel

L = _parity.L
O = _parity.O
F32 = np.float32

pytestmark = pytest.mark.gpu


def test_adjoint_matches_central_differences():
    n, batch, hfd = 32, 2048, 1e-3
    pr = problems.star_problem()
    g = mesh.uniform_grid(n)
    phi_np = O.perturb(np.asarray(pr["phi"](g.R.T), F32))
    ls = levelset.LevelSetGrid(g, phi_np, "cuda")
    pts = torch.as_tensor(g.R, device="cuda")
    h = np.array([g.dx, g.dy, g.dz], F32)
    lvl = FVLevel(ls, pr, pts, h)
    arch = nn.Arch(3, 32, 3, 32)
    p0 = nn.init_params(arch, 7)
    params = torch.as_tensor(p0, device="cuda")
    ids = ops.batch_ids(lvl.n, batch, epoch=0, batch_index=0, seed=5)
    ws = ops.StepWorkspace(arch, batch, lvl.max_jobs(batch), "cuda")
    ops.residual_forward(arch, params, lvl, ids, ws)
    grad = ops.residual_backward(arch, params, lvl, ids, ws).cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(11)
    idx = rng.choice(p0.size, 64, replace=False)

    def gpu_loss(p):
        loss, _, _ = ops.residual_forward(arch, torch.as_tensor(p, device="cuda"), lvl, ids, ws)
        return float(loss)

    fd32 = np.empty(idx.size)
    for k, i in enumerate(idx):
        pp, pm = p0.copy(), p0.copy()
        pp[i] += F32(hfd)
        pm[i] -= F32(hfd)
        fd32[k] = (gpu_loss(pp) - gpu_loss(pm)) / float(pp[i] - pm[i])
    scale = np.max(np.abs(grad[idx]))
    assert np.max(np.abs(fd32 - grad[idx])) <= 2e-2 * scale, np.max(np.abs(fd32 - grad[idx])) / scale

    # central differences of the oracle's loss in FP64 on the same batch
    sel = np.sort(ids.cpu().numpy())
    prob = L.Problem(phi_np, g.x, g.y, g.z, pr)
    rg = L.ResidualGeometry(prob, g.R[sel], h)
    a = L.Arch(3, 32, 3, 32)
    base = p0.astype(np.float64)

    def oracle_loss(p):
        return float(L.loss(torch.as_tensor(p), a, rg, torch.float64))

    fd64 = np.empty(idx.size)
    for k, i in enumerate(idx):
        pp, pm = base.copy(), base.copy()
        pp[i] += hfd
        pm[i] -= hfd
        fd64[k] = (oracle_loss(pp) - oracle_loss(pm)) / (2 * hfd)
    assert np.max(np.abs(fd64 - grad[idx])) <= 1e-3 * scale, np.max(np.abs(fd64 - grad[idx])) / scale
    assert np.linalg.norm(fd64 - grad[idx]) <= 1e-3 * np.linalg.norm(fd64)
