"""What the trained network gains over the method without it (the plain FV solve): the NBM
surrogate is trained on the residuals of the discretisation, BiCGSTAB solves the same FV
system, and both are evaluated off the grid against the exact solution.  Near the interface
the nodal Krylov solution, interpolated trilinearly, mixes the two sides of the jump; the network
is evaluated on the point's own side, so it is far more accurate there."""

import numpy as np
import pytest
import torch

from dips_gb300 import krylov, levelset, mesh, nn, ops, problems
from dips_gb300.records import FVLevel

pytestmark = pytest.mark.gpu


def test_trained_network_beats_interpolated_krylov_near_the_interface():
    pr = problems.sphere_problem()
    n = 32
    g = mesh.uniform_grid(n)
    ls = levelset.LevelSetGrid.from_callable(g, lambda r: levelset.perturb(pr["phi"](r)))
    lvl = FVLevel(ls, pr, torch.as_tensor(g.R, device="cuda"), np.array([g.dx, g.dy, g.dz], np.float32))
    # the plain method: BiCGSTAB on the same FV system
    shape = (n, n, n)
    kr = krylov.bicgstab(lvl, shape, max_iter=2000, rtol=1e-7, check_every=25)
    # the learned surrogate: NBM training with the fused step, full batch
    arch = nn.Arch(3, 32, 3, 32)
    params = torch.as_tensor(nn.init_params(arch, 42), device="cuda")
    opt = ops.AdamState(nn.n_params(arch), lr=1e-2, decay_rate=0.9)
    ws = ops.StepWorkspace(arch, lvl.n, lvl.max_jobs(lvl.n), "cuda")
    loss = torch.zeros((), dtype=torch.float64, device="cuda")
    first = None
    for it in range(3000):
        ops.train_step(arch, params, opt, lvl, None, ws, loss)
        if it == 0:
            first = float(loss)
    assert float(loss) < 1e-2 * first
    # off-grid comparison against the exact solution on the side each method sees
    rng = np.random.default_rng(7)
    q = torch.as_tensor(rng.uniform(-0.9, 0.9, (100000, 3)).astype(np.float32), device="cuda")
    phi_q = ls(q)
    qn = q.T.cpu().numpy()
    side = (phi_q >= 0).cpu().numpy()
    ex = torch.as_tensor(np.where(side, pr["u_p"](qn), pr["u_m"](qn)).astype(np.float32), device="cuda")
    u_nn = nn.mlp_eval(arch, params, q, phi_q)
    u_kr = levelset.LevelSetGrid(g, kr.x.reshape(-1).float())(q)
    near = phi_q.abs() < 2.0 * float(g.dx)
    scale = float(ex.abs().max())
    e_nn = float((u_nn - ex)[near].abs().max()) / scale
    e_kr = float((u_kr - ex)[near].abs().max()) / scale
    print(f"near the interface: network {e_nn:.4f}, interpolated Krylov {e_kr:.4f}")
    assert e_nn < 0.5 * e_kr, (e_nn, e_kr)
