"""Per-point residual records of one stencil spacing (one "level").

The reference recomputes the whole parameter-independent part of the residual --
cell decomposition, face areas, interface quadrature, regression extrapolation --
for every point at every step (solvers/poisson/discretization.py:299-519).  Here it
is computed once per (point, h) by the geometry kernels:

1. ``dips_geometry_classify``  flags and counts per point
2. ``dips_geometry_queries_ex``   the points where coefficient callables are needed
   (interface-triangle vertices, crossed stencil points, their projections r = s - phi n)
3. the host evaluates the user's coefficient callables at those points (torch, on the GPU)
4. ``dips_geometry_assemble_ex``  the residual of each point as an affine function of the
   network values at its jobs: r = nan_to_num((lhs0 + sum_j A_j u(x_j)) / diag) - rod
"""

from __future__ import annotations

import time

import numpy as np
import torch

from . import _lib, nonlinear
from .levelset import LevelSetGrid

F32 = np.float32


def eval_callable(fn, pts: torch.Tensor) -> torch.Tensor:
    """Evaluate a coefficient callable on points (M, 3); the callable sees r of shape (3, M)."""
    M = pts.shape[0]
    if M == 0:
        return torch.empty(0, dtype=torch.float32, device=pts.device)
    v = fn(pts.T)
    v = torch.as_tensor(v, dtype=torch.float32, device=pts.device)
    return torch.broadcast_to(v, (M,)).contiguous()


def _excl_scan(counts: torch.Tensor) -> torch.Tensor:
    c = counts.to(torch.int64)
    out = torch.zeros(c.numel() + 1, dtype=torch.int64, device=c.device)
    torch.cumsum(c, 0, out=out[1:])
    return out


class FVLevel:
    """Residual records of the points ``pts`` at stencil spacing ``h`` (device tensors)."""

    def __init__(self, ls: LevelSetGrid, coeff_fns: dict, pts: torch.Tensor, h, keep_geometry=False, profile=False):
        lib = _lib.load()
        dev = pts.device
        # profile: host seconds per set-up phase (device synchronised at each boundary)
        self.timings = {} if profile else None
        _t = [time.perf_counter()]

        def mark(name):
            if profile:
                torch.cuda.synchronize(dev)
                now = time.perf_counter()
                self.timings[name] = now - _t[0]
                _t[0] = now

        mark("start")
        self.ls = ls
        self.pts = pts.to(torch.float32).contiguous()
        n = self.pts.shape[0]
        self.n = n
        self.h = np.asarray(h, F32).reshape(3)
        hc = (_lib.c_f32 * 3)(*[float(v) for v in self.h])
        st = _lib.stream_handle()
        i32 = dict(dtype=torch.int32, device=dev)
        flags = torch.empty(n, **i32)
        n_tri = torch.empty(n, **i32)
        n_xs = torch.empty(n, **i32)
        cap = torch.empty(n, **i32)
        P = _lib.ptr
        _lib.check(
            lib.dips_geometry_classify(ls.desc, P(self.pts), n, hc, P(flags), P(n_tri), P(n_xs), P(cap), st),
            "dips_geometry_classify",
        )
        mark("classify")
        tri_off = _excl_scan(n_tri)
        xs_off = _excl_scan(n_xs)
        self.job_off = _excl_scan(cap)
        n_tri_tot = int(tri_off[-1])
        n_xs_tot = int(xs_off[-1])
        self.n_jobs_cap = int(self.job_off[-1])
        f32 = dict(dtype=torch.float32, device=dev)
        tri_pts = torch.empty(max(3 * n_tri_tot, 1), 3, **f32)
        xs_pts = torch.empty(max(n_xs_tot, 1), 3, **f32)
        xr_pts = torch.empty(max(n_xs_tot, 1), 3, **f32)
        # the points next to the interface are listed in scratch and run together (queries, and the
        # second launch of the assembly)
        scratch = torch.empty(max(int(lib.dips_geometry_assemble_scratch_bytes(n)), 4), dtype=torch.uint8, device=dev)
        _lib.check(
            lib.dips_geometry_queries_ex(ls.desc, P(self.pts), n, hc, P(flags), P(tri_off), P(xs_off), P(tri_pts),
                                         P(xs_pts), P(xr_pts), P(scratch), scratch.numel(), st),
            "dips_geometry_queries_ex",
        )
        tri_pts = tri_pts[: 3 * n_tri_tot]
        xs_pts = xs_pts[:n_xs_tot]
        xr_pts = xr_pts[:n_xs_tot]
        mark("scans_and_queries")

        # ---- coefficient callables (reference semantics: evaluated at exactly these points)
        fn = coeff_fns
        half = torch.tensor(0.5, dtype=torch.float32, device=dev)
        hv = torch.as_tensor(self.h, device=dev)
        offs = torch.zeros(6, 3, **f32)
        for a in range(3):
            offs[2 * a, a] = -hv[a]
            offs[2 * a + 1, a] = hv[a]
        offs = half * offs
        faces = (self.pts[:, None, :] + offs[None]).reshape(-1, 3)
        self._face_offs = offs
        vals = {}
        vals["mu_m_face"] = eval_callable(fn["mu_m"], faces)
        vals["mu_p_face"] = eval_callable(fn["mu_p"], faces)
        del faces
        for name in ("k_m", "k_p", "f_m", "f_p", "g"):
            vals[name] = eval_callable(fn[name], self.pts)
        vals["beta_tri"] = eval_callable(fn["beta"], tri_pts)
        vals["mu_m_s"] = eval_callable(fn["mu_m"], xs_pts)
        vals["mu_p_s"] = eval_callable(fn["mu_p"], xs_pts)
        vals["alpha_r"] = eval_callable(fn["alpha"], xr_pts)
        vals["beta_r"] = eval_callable(fn["beta"], xr_pts)
        vals["mu_m_r"] = eval_callable(fn["mu_m"], xr_pts)
        vals["mu_p_r"] = eval_callable(fn["mu_p"], xr_pts)
        beta0 = float(eval_callable(fn["beta"], torch.zeros(1, 3, **f32))[0])
        for k, v in vals.items():
            if v.numel() == 0:
                vals[k] = torch.zeros(1, **f32)
        co = _lib.CoeffsT(*[P(vals[k]) for k, _ in _lib.CoeffsT._fields_[:-1]], beta0)
        mark("coefficient_callables")

        self.lhs0 = torch.empty(n, **f32)
        self.diag = torch.empty(n, **f32)
        self.rod = torch.empty(n, **f32)
        self.cnt = torch.empty(n, **i32)
        self.cnt_m = torch.empty(n, **i32)
        self.job_code = torch.empty(max(self.n_jobs_cap, 1), dtype=torch.int16, device=dev)
        self.job_A = torch.zeros(max(self.n_jobs_cap, 1), **f32)
        self.coeff26 = torch.empty(n, 26, **f32) if keep_geometry else None
        self.beta_int = torch.empty(n, **f32) if keep_geometry else None
        # nonlinear operators (``nl_m``/``nl_p`` in the coefficient dict): their arguments' records
        self.nl = (nonlinear.resolve(coeff_fns.get("nl_m")), nonlinear.resolve(coeff_fns.get("nl_p")))
        has_nl = not (nonlinear.is_zero(self.nl[0]) and nonlinear.is_zero(self.nl[1]))
        self.nl_pt = torch.empty(max(n, 1), 4, **f32) if has_nl else None
        self.nl_w = torch.zeros(max(self.n_jobs_cap, 1), 2, **f32) if has_nl else None
        _lib.check(
            lib.dips_geometry_assemble_ex(ls.desc, P(self.pts), n, hc, P(flags), P(tri_off), P(xs_off),
                                          P(self.job_off), co, P(self.lhs0), P(self.diag), P(self.rod), P(self.cnt),
                                          P(self.cnt_m), P(self.job_code), P(self.job_A), P(self.coeff26),
                                          P(self.beta_int), P(self.nl_pt), P(self.nl_w), P(scratch), scratch.numel(),
                                          st),
            "dips_geometry_assemble_ex",
        )
        mark("assemble")
        self.flags = flags if keep_geometry else None
        self.n_tri, self.n_xs = (n_tri, n_xs) if keep_geometry else (None, None)
        self._vals = vals if keep_geometry else None
        # what the coefficient tangent needs: the query points and offsets, the coefficients
        self._geo = (tri_off, xs_off, tri_pts, xs_pts, xr_pts, co, beta0) if keep_geometry else None
        self.n_jobs = int(self.cnt.sum())
        self.max_cnt = int(self.cnt.max()) if n else 0
        self.desc = _lib.RecordsT(
            P(self.pts), n, (_lib.c_f32 * 3)(*[float(v) for v in self.h]), P(self.lhs0), P(self.diag), P(self.rod),
            P(self.cnt), P(self.cnt_m), P(self.job_off), P(self.job_code), P(self.job_A), P(self.coeff26), None,
        )
        if has_nl:
            self.desc.nl_pt = P(self.nl_pt)
            self.desc.nl_w = P(self.nl_w)
            self.desc.nl_kind = (_lib.c_i32 * 2)(self.nl[0].kind, self.nl[1].kind)
            self.desc.nl_c = (_lib.c_f32 * 2)(self.nl[0].c, self.nl[1].c)
        # each bulk point's 64-byte record, packed once so that a step reads it in one piece
        self.bulk_rec = torch.empty(max(n, 1), 16, **f32)
        if n:
            _lib.check(lib.dips_pack_bulk_records(self.desc, P(self.bulk_rec), st), "dips_pack_bulk_records")
        self.desc.bulk_rec = P(self.bulk_rec)
        mark("pack_bulk_records")

    def coefficient_tangent(self, dfns: dict) -> "TangentRecords":
        """Derivative of the records along a direction in coefficient space.

        ``dfns`` maps coefficient names (mu_m, mu_p, k_m, k_p, f_m, f_p, g, alpha, beta) to
        callables r -> the derivative of that coefficient at r along the direction; absent names
        do not change.  ``{"mu_p": lambda r: 1.0}`` is d/d mu+ of a constant mu+.  Needs a level
        built with keep_geometry=True."""
        if self._geo is None:
            raise ValueError("coefficient_tangent needs FVLevel(..., keep_geometry=True)")
        unknown = set(dfns) - {"mu_m", "mu_p", "k_m", "k_p", "f_m", "f_p", "g", "alpha", "beta"}
        if unknown:
            raise ValueError(f"unknown coefficient names {sorted(unknown)}")
        lib = _lib.load()
        tri_off, xs_off, tri_pts, xs_pts, xr_pts, co, _ = self._geo
        faces = (self.pts[:, None, :] + self._face_offs[None]).reshape(-1, 3)
        where = {"mu_m_face": ("mu_m", faces), "mu_p_face": ("mu_p", faces), "k_m": ("k_m", self.pts),
                 "k_p": ("k_p", self.pts), "f_m": ("f_m", self.pts), "f_p": ("f_p", self.pts), "g": ("g", self.pts),
                 "beta_tri": ("beta", tri_pts), "mu_m_s": ("mu_m", xs_pts), "mu_p_s": ("mu_p", xs_pts),
                 "alpha_r": ("alpha", xr_pts), "beta_r": ("beta", xr_pts), "mu_m_r": ("mu_m", xr_pts),
                 "mu_p_r": ("mu_p", xr_pts)}
        keep = {}
        ptrs = []
        for field, _ in _lib.CoeffsT._fields_[:-1]:
            name, at = where[field]
            if name in dfns and at.shape[0] > 0:
                keep[field] = eval_callable(dfns[name], at)
                ptrs.append(_lib.ptr(keep[field]))
            else:
                ptrs.append(None)
        dco = _lib.CoeffsT(*ptrs, 0.0)
        t = TangentRecords(self)
        P = _lib.ptr
        _lib.check(
            lib.dips_geometry_assemble_tangent(self.ls.desc, P(self.pts), self.n, self._hc(), P(self.flags),
                                               P(tri_off), P(xs_off), P(self.job_off), co, dco, P(t.lhs0),
                                               P(t.diag), P(t.rod), P(t.job_A), _lib.stream_handle()),
            "dips_geometry_assemble_tangent",
        )
        return t

    def _hc(self):
        return (_lib.c_f32 * 3)(*[float(v) for v in self.h])

    def max_jobs(self, batch: int, distinct: bool = True) -> int:
        """Upper bound of the jobs of a batch of ``batch`` points (distinct points: <= all jobs)."""
        bound = batch * self.max_cnt
        return min(bound, self.n_jobs) if distinct else bound


class TangentRecords:
    """d lhs0, d diag, d rod (per point) and d job_A (per job) of a level along a coefficient
    direction; ``desc`` is the level's record descriptor with these four arrays in place."""

    def __init__(self, level: FVLevel):
        f32 = dict(dtype=torch.float32, device=level.pts.device)
        n = level.n
        self.level = level
        self.lhs0 = torch.zeros(n, **f32)
        self.diag = torch.zeros(n, **f32)
        self.rod = torch.zeros(n, **f32)
        self.job_A = torch.zeros(level.job_A.numel(), **f32)
        d = level.desc
        P = _lib.ptr
        self.desc = _lib.RecordsT(d.pts, d.n_pts, d.h, P(self.lhs0), P(self.diag), P(self.rod), d.cnt, d.cnt_m,
                                  d.job_off, d.job_code, P(self.job_A), d.coeff26, None)
