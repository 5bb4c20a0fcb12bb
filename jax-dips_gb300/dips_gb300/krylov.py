"""Plain method: the FV system of a nodal vector and a matrix-free BiCGSTAB on it.

The reference defines the operator (``Trainer.residual_vector``, solvers/poisson/
trainer.py:883-890 over compute_Ax_and_b_discrete_fn, discretization.py:522-741) but has
no Krylov loop; this module supplies one on the same per-point FV records as the NBM path.
"""

from __future__ import annotations

import dataclasses

import torch

from . import _lib
from .records import FVLevel


@dataclasses.dataclass
class KrylovResult:
    x: torch.Tensor
    iterations: int
    target_iteration: int
    breakdown: bool
    rel_residual: float
    rel_linf: float


def _grid_shape(level: FVLevel, shape):
    nx, ny, nz = (int(s) for s in shape)
    if nx * ny * nz != level.n:
        raise ValueError("the records' points must be the grid nodes in C order")
    return nx, ny, nz


def fv_residual(level: FVLevel, shape, u: torch.Tensor, linear_only=False) -> torch.Tensor:
    """K u - b (or K u) for a nodal vector u on the records' grid."""
    lib = _lib.load()
    nx, ny, nz = _grid_shape(level, shape)
    u = u.to(torch.float32).contiguous()
    out = torch.empty_like(u)
    _lib.check(lib.dips_fv_residual(level.desc, nx, ny, nz, _lib.ptr(u), int(bool(linear_only)), _lib.ptr(out),
                                    _lib.stream_handle()), "dips_fv_residual")
    return out


def bicgstab(level: FVLevel, shape, x0=None, u_exact=None, max_iter=5000, rtol=1e-6, check_every=10,
             target_rel_linf=0.0, workspace=None) -> KrylovResult:
    lib = _lib.load()
    nx, ny, nz = _grid_shape(level, shape)
    dev = level.pts.device
    x = torch.zeros(level.n, dtype=torch.float32, device=dev) if x0 is None else x0.clone().to(torch.float32)
    nbytes = int(lib.dips_bicgstab_workspace_bytes(level.n))
    ws = workspace if workspace is not None and workspace.numel() >= nbytes else torch.empty(
        nbytes, dtype=torch.uint8, device=dev)
    ex = None if u_exact is None else u_exact.to(torch.float32).contiguous()
    st = _lib.KrylovStatsT()
    _lib.check(lib.dips_bicgstab(level.desc, nx, ny, nz, _lib.ptr(x), _lib.ptr(ex), int(max_iter), float(rtol),
                                 int(check_every), float(target_rel_linf), _lib.ptr(ws), ws.numel(), st,
                                 _lib.stream_handle()), "dips_bicgstab")
    return KrylovResult(x, st.iterations, st.target_iteration, bool(st.breakdown), st.rel_residual, st.rel_linf)
