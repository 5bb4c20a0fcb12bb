"""Level-set grid on the device and its trilinear interpolant.

The level set is sampled on ``lvl_gstate`` and interpolated trilinearly with the
reference's ``multilinear_interpolation`` semantics (domain/interpolate.py:906-1021):
a ghost layer of linear extrapolation is added around the samples by
``dips_phi_ghost_layer`` and queries go through ``dips_phi_trilinear``.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .mesh import GridState

F32 = np.float32


def perturb(phi: torch.Tensor) -> torch.Tensor:
    """``perturb_level_set_fn`` (geometry/level_set.py:34-48): phi + sign_pm(phi)*1e-10."""
    sgn = torch.sign(torch.sign(phi) - 0.5)
    return phi + sgn * 1.0e-10


def ghost_coords(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a, F32)
    out = np.zeros(a.shape[0] + 2, F32)
    out[1:-1] = a
    out[0] = a[0] - (a[1] - a[0])
    out[-1] = a[-1] + (a[-1] - a[-2])
    return out


class LevelSetGrid:
    """Ghosted level-set samples resident in HBM plus the C-ABI descriptor."""

    def __init__(self, gstate: GridState, phi_values, device="cuda"):
        lib = _lib.load()
        self.gstate = gstate
        nx, ny, nz = gstate.x.shape[0], gstate.y.shape[0], gstate.z.shape[0]
        phi = torch.as_tensor(np.asarray(phi_values, F32) if not torch.is_tensor(phi_values) else phi_values)
        phi = phi.to(device=device, dtype=torch.float32).contiguous().reshape(-1)
        if phi.numel() != nx * ny * nz:
            raise ValueError(f"level set has {phi.numel()} samples, grid has {nx * ny * nz}")
        self.phi = phi
        self.gh = torch.empty((nx + 2) * (ny + 2) * (nz + 2), dtype=torch.float32, device=device)
        self.xg = torch.as_tensor(ghost_coords(gstate.x), device=device)
        self.yg = torch.as_tensor(ghost_coords(gstate.y), device=device)
        self.zg = torch.as_tensor(ghost_coords(gstate.z), device=device)
        _lib.check(
            lib.dips_phi_ghost_layer(_lib.ptr(self.phi), nx, ny, nz, _lib.ptr(self.gh), _lib.stream_handle()),
            "dips_phi_ghost_layer",
        )
        self.desc = _lib.LevelSetT(
            _lib.ptr(self.gh), _lib.ptr(self.xg), _lib.ptr(self.yg), _lib.ptr(self.zg), nx, ny, nz,
            float(gstate.xmin()), float(gstate.xmax()), float(gstate.ymin()), float(gstate.ymax()),
            float(gstate.zmin()), float(gstate.zmax()),
        )

    @classmethod
    def from_callable(cls, gstate: GridState, phi_fn, device="cuda"):
        """Sample a level-set callable ``phi_fn(r)`` (r of shape (3, M)) on the grid nodes."""
        R = torch.as_tensor(gstate.R, device=device)
        vals = torch.as_tensor(phi_fn(R.T), device=device, dtype=torch.float32)
        return cls(gstate, vals.reshape(-1), device)

    def quadratic(self, pts: torch.Tensor) -> torch.Tensor:
        """Non-oscillatory quadratic interpolation at points (n, 3) (interpolate.py:572-759)."""
        lib = _lib.load()
        pts = pts.to(torch.float32).contiguous()
        out = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
        _lib.check(
            lib.dips_phi_quadratic(self.desc, _lib.ptr(pts), pts.shape[0], _lib.ptr(out), _lib.stream_handle()),
            "dips_phi_quadratic",
        )
        return out

    def __call__(self, pts: torch.Tensor) -> torch.Tensor:
        """Trilinear interpolation at points (n, 3)."""
        lib = _lib.load()
        pts = pts.to(torch.float32).contiguous()
        out = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
        _lib.check(
            lib.dips_phi_trilinear(self.desc, _lib.ptr(pts), pts.shape[0], _lib.ptr(out), _lib.stream_handle()),
            "dips_phi_trilinear",
        )
        return out
