"""Shared set-up for the parity tests: the same synthetic inputs fed to the CUDA path
(through the C ABI) and to the CPU oracle."""

from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("jax-dips_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

import nbm_loss as L  # noqa: E402
import nbm_oracle as O  # noqa: E402
from dips_gb300 import mesh, problems  # noqa: E402

F32 = np.float32


def make_problem(name):
    if name == "sphere":
        return problems.sphere_problem()
    if name == "star":
        return problems.star_problem()
    raise KeyError(name)


class Case:
    """A grid problem at one stencil level with a fixed parameter vector."""

    def __init__(self, name="sphere", n=16, arch=(1, 1, 2, 10), level=0, seed=0, batch=None, batch_seed=0,
                 fns=None, phi=None, params=None, ids=None):
        self.name = name
        self.fns = fns if fns is not None else make_problem(name)
        self.grid = mesh.uniform_grid(n)
        g = self.grid
        self.phi = phi if phi is not None else O.perturb(np.asarray(self.fns["phi"](g.R.T), F32))
        self.h = np.array([g.dx, g.dy, g.dz], F32) * F32(0.5**level)
        self.arch = L.Arch(*arch)
        self.params = params if params is not None else L.init_params(self.arch, seed)
        self.pts = g.R
        self.batch = None
        if ids is not None:
            self.batch = np.asarray(ids, np.int32)
        elif batch is not None:
            rng = np.random.default_rng(batch_seed)
            self.batch = np.sort(rng.choice(g.R.shape[0], batch, replace=False)).astype(np.int32)
        self._rg = None
        self._level = None

    # ---------------- oracle side
    @property
    def oracle_problem(self):
        g = self.grid
        return L.Problem(self.phi, g.x, g.y, g.z, self.fns)

    def oracle_geometry(self):
        if self._rg is None:
            pts = self.pts if self.batch is None else self.pts[self.batch]
            self._rg = L.ResidualGeometry(self.oracle_problem, pts, self.h)
        return self._rg

    def oracle_loss_grad(self, dtype=None):
        import torch

        dtype = dtype or torch.float32
        return L.loss_and_grad(self.params, self.arch, self.oracle_geometry(), dtype)

    def oracle_residual(self, dtype=None):
        import torch

        dtype = dtype or torch.float32
        return L.residual(torch.tensor(self.params).to(dtype), self.arch, self.oracle_geometry(), dtype).numpy()

    # ---------------- CUDA side
    def gpu_level(self):
        import torch

        from dips_gb300 import levelset, records

        if self._level is None:
            ls = levelset.LevelSetGrid(self.grid, self.phi)
            pts = torch.as_tensor(self.pts, device="cuda")
            self._ls = ls
            self._level = records.FVLevel(ls, self.fns, pts, self.h, keep_geometry=True)
        return self._level

    def gpu_arch(self):
        from dips_gb300.nn import Arch

        a = self.arch
        return Arch(a.m_layers, a.m_width, a.p_layers, a.p_width, a.pre_layers, a.pre_width, a.pre_scaling)

    def gpu_batch_ids(self):
        import torch

        return None if self.batch is None else torch.as_tensor(self.batch, device="cuda")

    def gpu_loss_grad(self):
        import torch

        from dips_gb300 import ops

        lvl = self.gpu_level()
        params = torch.as_tensor(self.params, device="cuda")
        ids = self.gpu_batch_ids()
        loss, _, ws = ops.residual_forward(self.gpu_arch(), params, lvl, ids)
        grad = ops.residual_backward(self.gpu_arch(), params, lvl, ids, ws)
        torch.cuda.synchronize()
        return float(loss), grad.cpu().numpy()

    def gpu_residual(self):
        import torch

        from dips_gb300 import ops

        lvl = self.gpu_level()
        params = torch.as_tensor(self.params, device="cuda")
        _, res, _ = ops.residual_forward(self.gpu_arch(), params, lvl, self.gpu_batch_ids(), want_residual=True)
        return res.cpu().numpy()


def build_case(name="sphere", n=16, arch=(1, 1, 2, 10), level=0, **kw):
    return Case(name, n, arch, level, **kw)


GOLDEN = os.path.join(ROOT, "tests", "golden")


def reference_fixtures(kind="loss"):
    """Names of the fixtures written by the reference's own code (tests/golden/ref_*.npz):
    kind "loss" for the network residual cases, "fvop" for the discrete operator of a nodal vector
    (the batch-layout and interpolant fixtures, ``ref_dataset_*`` and ``ref_interp_*``, are neither)."""
    names = sorted(f[4:-4] for f in os.listdir(GOLDEN) if f.startswith("ref_") and f.endswith(".npz"))
    names = [k for k in names if not k.startswith(("dataset_", "interp_"))]
    return [k for k in names if k.startswith("fvop_") == (kind == "fvop")]


def load_reference_fixture(key):
    return dict(np.load(os.path.join(GOLDEN, f"ref_{key}.npz")))


def reference_case(key):
    """The parity case of a reference fixture: its problem, grid, level, network, phi samples,
    parameters and batch, fed unchanged to the oracle and to the CUDA path."""
    from golden import make_reference_golden as M

    fx = load_reference_fixture(key)
    prob = str(fx["problem"])
    return Case(prob, int(fx["n"]), tuple(int(v) for v in fx["arch"]), int(fx["level"]), fns=M.problem(prob),
                phi=fx["phi"], params=fx["params"], ids=fx["ids"]), fx
