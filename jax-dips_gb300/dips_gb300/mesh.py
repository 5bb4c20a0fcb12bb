"""Grid state and mesh construction (mirror of jax_dips/domain/mesh.py).

``GridState`` keeps the reference's fields (x, y, z, R, dx, dy, dz and the six
boundary point sets, domain/mesh.py:39-89) as float32 numpy arrays, and
``construct(3)`` returns ``(init_fn, point_fn)`` like the reference
(domain/mesh.py:92-176): points are the 'ij' meshgrid flattened in C order.
"""

from __future__ import annotations

import dataclasses

import numpy as np

F32 = np.float32


def linspace_f32(start, stop, num):
    """``jnp.linspace(start, stop, num, dtype=f32)`` as jax evaluates it with x64 off:
    ``start*(1-t) + stop*t`` with ``t = i/(num-1)`` in float32, last entry ``stop``."""
    start, stop = F32(start), F32(stop)
    if num == 1:
        return np.array([start], F32)
    div = num - 1
    t = (np.arange(div, dtype=F32) / F32(div)).astype(F32)
    out = (start * (F32(1.0) - t) + stop * t).astype(F32)
    return np.concatenate([out, np.array([stop], F32)]).astype(F32)


@dataclasses.dataclass
class GridState:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    R: np.ndarray
    dx: float
    dy: float
    dz: float
    R_xmin_boundary: np.ndarray
    R_xmax_boundary: np.ndarray
    R_ymin_boundary: np.ndarray
    R_ymax_boundary: np.ndarray
    R_zmin_boundary: np.ndarray
    R_zmax_boundary: np.ndarray

    def shape(self):
        return self.x.shape + self.y.shape + self.z.shape

    def xmin(self):
        return F32(self.x.min())

    def xmax(self):
        return F32(self.x.max())

    def ymin(self):
        return F32(self.y.min())

    def ymax(self):
        return F32(self.y.max())

    def zmin(self):
        return F32(self.z.min())

    def zmax(self):
        return F32(self.z.max())

    def base_level(self):
        return int(np.log2(len(self.R) ** (1.0 / 3.0)))


def construct(dimension: int):
    if dimension != 3:
        raise NotImplementedError("only the 3-D mesh is on this path")

    def init_fn_3d(x, y, z):
        x, y, z = (np.asarray(a, F32) for a in (x, y, z))
        dx, dy, dz = F32(x[1] - x[0]), F32(y[1] - y[0]), F32(z[1] - z[0])
        X_, Y_, Z_ = np.meshgrid(x, y, z, indexing="ij")
        R = np.column_stack((X_.ravel(), Y_.ravel(), Z_.ravel())).astype(F32)

        def face(sl):
            return np.column_stack((X_[sl].ravel(), Y_[sl].ravel(), Z_[sl].ravel())).astype(F32)

        return GridState(
            x, y, z, R, dx, dy, dz,
            face((0, slice(None), slice(None))), face((-1, slice(None), slice(None))),
            face((slice(None), 0, slice(None))), face((slice(None), -1, slice(None))),
            face((slice(None), slice(None), 0)), face((slice(None), slice(None), -1)),
        )

    def point3d_at(gstate, idx):
        return [gstate.x[idx[0]], gstate.y[idx[1]], gstate.z[idx[2]]]

    return init_fn_3d, point3d_at


def uniform_grid(n, lo=-1.0, hi=1.0):
    """GridState of an n^3 grid over [lo, hi]^3 built with the jax linspace."""
    init_fn, _ = construct(3)
    a = linspace_f32(lo, hi, n)
    return init_fn(a, a, a)
