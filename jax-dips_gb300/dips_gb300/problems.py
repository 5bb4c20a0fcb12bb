"""Manufactured interface problems used by the tests and the benchmark.

Each problem is a dict of coefficient callables in the shape the reference's
``trainer.setup`` takes (solvers/poisson/trainer.py:980-994), except that a
callable receives a whole coordinate array ``r`` of shape (3, M) -- a numpy
array or a torch tensor -- and returns shape (M,).  ``x, y, z = r`` and
``r[0]`` work as in the reference's per-point callables
(tests/confs/experiment_configs.py).

Sign conventions follow the reference's FV residual
(solvers/poisson/discretization.py:403-408): the PDE is
``-div(mu grad u) + k u = f`` and the flux jump enters the right-hand side as
``+ int_Gamma beta dA`` with ``beta = -(mu+ d_n u+ - mu- d_n u-)``, n the unit
normal pointing from Omega^- (phi < 0) into Omega^+ (see
tests/confs/experiment_configs.py:84-96).  ``alpha = u+ - u-``.
"""

from __future__ import annotations

import math

import numpy as np

try:  # torch is optional for the numpy-only users of this module
    import torch
except Exception:  # pragma: no cover
    torch = None


# ----------------------------------------------------------------------------------------
# array-namespace helpers: the same callable runs on numpy (CPU) or torch (GPU) arrays
# ----------------------------------------------------------------------------------------
def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


class _NS:
    def __init__(self, like):
        self.t = _is_torch(like)
        self.like = like

    def __getattr__(self, name):
        mod = torch if self.t else np
        alias = {"arccos": "acos", "arctan2": "atan2"} if self.t else {}
        return getattr(mod, alias.get(name, name))

    def full(self, value):
        if self.t:
            return torch.full_like(self.like, float(value))
        return np.full_like(self.like, value)

    def maximum(self, a, b):
        if self.t:
            return torch.clamp(a, min=b) if not _is_torch(b) else torch.maximum(a, b)
        return np.maximum(a, b)

    def safe_div(self, a, b):
        """a / b with b == 0 replaced by 1 (so 0/0 -> 0)."""
        if self.t:
            return a / torch.where(b == 0, torch.ones_like(b), b)
        return a / np.where(b == 0, np.ones_like(b), b)

    def ieee_div(self, a, b):
        """a / b with IEEE results at b == 0 (0/0 -> NaN) and no numpy warning for them."""
        if self.t:
            return a / b
        with np.errstate(invalid="ignore", divide="ignore"):
            return a / b


def _xyz(r):
    return r[0], r[1], r[2], _NS(r[0])


# ----------------------------------------------------------------------------------------
# sphere (configs 1 and 2): phi = |x| - 0.5
# ----------------------------------------------------------------------------------------
def sphere_problem(mu_m=1.0, mu_p=10.0):
    """Sphere interface, u- = sin x cos y e^z, u+ = x^2+y^2+z^2, mu-=1, mu+=10, k=0."""

    def phi(r):
        x, y, z, xp = _xyz(r)
        return xp.sqrt(x * x + y * y + z * z) - 0.5

    def u_m(r):
        x, y, z, xp = _xyz(r)
        return xp.sin(x) * xp.cos(y) * xp.exp(z)

    def u_p(r):
        x, y, z, xp = _xyz(r)
        return x * x + y * y + z * z

    def grad_u_m(r):
        x, y, z, xp = _xyz(r)
        e = xp.exp(z)
        return (xp.cos(x) * xp.cos(y) * e, -xp.sin(x) * xp.sin(y) * e, xp.sin(x) * xp.cos(y) * e)

    def normal(r):
        x, y, z, xp = _xyz(r)
        n = xp.sqrt(x * x + y * y + z * z)
        return xp.safe_div(x, n), xp.safe_div(y, n), xp.safe_div(z, n)

    def beta(r):
        x, y, z, xp = _xyz(r)
        nx, ny, nz = normal(r)
        gm = grad_u_m(r)
        dn_up = 2.0 * x * nx + 2.0 * y * ny + 2.0 * z * nz
        dn_um = gm[0] * nx + gm[1] * ny + gm[2] * nz
        return -(mu_p * dn_up - mu_m * dn_um)

    def f_m(r):  # -mu- lap(u-) ; lap(sin x cos y e^z) = -sin x cos y e^z
        return mu_m * u_m(r)

    def f_p(r):
        x, y, z, xp = _xyz(r)
        return xp.full(-6.0 * mu_p)

    return _assemble(phi, u_m, u_p, lambda r: _xyz(r)[3].full(mu_m), lambda r: _xyz(r)[3].full(mu_p),
                     lambda r: _xyz(r)[3].full(0.0), lambda r: _xyz(r)[3].full(0.0), f_m, f_p, beta)


# ----------------------------------------------------------------------------------------
# star (config 3): phi = r - 0.5 - 0.15 sin(5 theta) cos(3 varphi)
# ----------------------------------------------------------------------------------------
def star_problem():
    """Star interface, variable mu, k+ = 1; u- = exp(-|x|^2), u+ = cos(x+y+z)."""

    def _angles(r):
        x, y, z, xp = _xyz(r)
        rr = xp.sqrt(x * x + y * y + z * z)
        cz = xp.clip(xp.safe_div(z, rr), -1.0, 1.0)
        theta = xp.arccos(cz)
        vphi = xp.arctan2(y, x)
        return rr, theta, vphi

    def phi(r):
        rr, th, vp = _angles(r)
        xp = _xyz(r)[3]
        return rr - 0.5 - 0.15 * xp.sin(5.0 * th) * xp.cos(3.0 * vp)

    def grad_phi(r):
        x, y, z, xp = _xyz(r)
        rr, th, vp = _angles(r)
        rho2 = x * x + y * y
        rho = xp.sqrt(rho2)
        r2 = rr * rr
        A = -0.15 * 5.0 * xp.cos(5.0 * th) * xp.cos(3.0 * vp)  # d phi / d theta
        B = 0.15 * 3.0 * xp.sin(5.0 * th) * xp.sin(3.0 * vp)  # d phi / d varphi
        dth_dx = xp.safe_div(x * z, r2 * rho)
        dth_dy = xp.safe_div(y * z, r2 * rho)
        dth_dz = xp.safe_div(-rho, r2)
        dvp_dx = xp.safe_div(-y, rho2)
        dvp_dy = xp.safe_div(x, rho2)
        gx = xp.safe_div(x, rr) + A * dth_dx + B * dvp_dx
        gy = xp.safe_div(y, rr) + A * dth_dy + B * dvp_dy
        gz = xp.safe_div(z, rr) + A * dth_dz
        return gx, gy, gz

    def mu_m(r):
        x, y, z, xp = _xyz(r)
        return 1.0 + 0.5 * xp.sin(x * y)

    def mu_p(r):
        x, y, z, xp = _xyz(r)
        return 20.0 + 5.0 * xp.cos(z)

    def u_m(r):
        x, y, z, xp = _xyz(r)
        return xp.exp(-(x * x + y * y + z * z))

    def u_p(r):
        x, y, z, xp = _xyz(r)
        return xp.cos(x + y + z)

    def f_m(r):
        x, y, z, xp = _xyz(r)
        rr2 = x * x + y * y + z * z
        e = xp.exp(-rr2)
        return 2.0 * x * y * xp.cos(x * y) * e - (1.0 + 0.5 * xp.sin(x * y)) * (4.0 * rr2 - 6.0) * e

    def f_p(r):
        x, y, z, xp = _xyz(r)
        s = x + y + z
        return -5.0 * xp.sin(z) * xp.sin(s) + 3.0 * (20.0 + 5.0 * xp.cos(z)) * xp.cos(s) + xp.cos(s)

    def beta(r):
        x, y, z, xp = _xyz(r)
        gx, gy, gz = grad_phi(r)
        gn = xp.sqrt(gx * gx + gy * gy + gz * gz)
        nx, ny, nz = xp.safe_div(gx, gn), xp.safe_div(gy, gn), xp.safe_div(gz, gn)
        e = xp.exp(-(x * x + y * y + z * z))
        gum = (-2.0 * x * e, -2.0 * y * e, -2.0 * z * e)
        sn = -xp.sin(x + y + z)
        dn_up = sn * (nx + ny + nz)
        dn_um = gum[0] * nx + gum[1] * ny + gum[2] * nz
        return -(mu_p(r) * dn_up - mu_m(r) * dn_um)

    return _assemble(phi, u_m, u_p, mu_m, mu_p, lambda r: _xyz(r)[3].full(0.0),
                     lambda r: _xyz(r)[3].full(1.0), f_m, f_p, beta)


# ----------------------------------------------------------------------------------------
# the reference's own manufactured problems (tests/confs/experiment_configs.py)
# ----------------------------------------------------------------------------------------
def reference_sphere_problem():
    """``sphere()`` of tests/confs/experiment_configs.py:21-186: phi = |x| - 0.5,
    u- = e^z, u+ = sin y cos x, mu- = y^2 ln(x + 2) + 4, mu+ = e^-z, k = 0, g = u+,
    f from its hand-written f_m_fn/f_p_fn (:158-172), beta = -(mu+ grad u+ - mu- grad u-) . grad phi
    (:84-96, grad phi not normalised; it is a unit vector for this phi).  mu- > mu+ everywhere in
    [-1, 1]^3, so every interface point takes the reference's mu- > mu+ extrapolation branch
    (solvers/poisson/discretization.py:464-486)."""

    def phi(r):
        x, y, z, xp = _xyz(r)
        return xp.sqrt(x * x + y * y + z * z) - 0.5

    def u_m(r):
        x, y, z, xp = _xyz(r)
        return xp.exp(z)

    def u_p(r):
        x, y, z, xp = _xyz(r)
        return xp.sin(y) * xp.cos(x)

    def mu_m(r):
        x, y, z, xp = _xyz(r)
        return y * y * xp.log(x + 2.0) + 4.0

    def mu_p(r):
        x, y, z, xp = _xyz(r)
        return xp.exp(-1.0 * z)

    def beta(r):
        # grad phi = x / |x|: 0/0 = NaN at the origin, as jax.grad of the reference's phi gives
        # there; the reference integrates beta at the origin (its zero-padding triangles), so a
        # crossed cell's interface integral, and then its rhs/diag, come out NaN -> 0
        x, y, z, xp = _xyz(r)
        n = xp.sqrt(x * x + y * y + z * z)
        nx, ny, nz = xp.ieee_div(x, n), xp.ieee_div(y, n), xp.ieee_div(z, n)
        mp, mm = mu_p(r), mu_m(r)
        gpx, gpy = -xp.sin(y) * xp.sin(x), xp.cos(y) * xp.cos(x)
        gmz = xp.exp(z)
        return ((mp * gpx) * nx + (mp * gpy) * ny + (0.0 - mm * gmz) * nz) * (-1.0)

    def f_m(r):
        x, y, z, xp = _xyz(r)
        return -1.0 * xp.exp(z) * (y * y * xp.log(x + 2.0) + 4.0)

    def f_p(r):
        x, y, z, xp = _xyz(r)
        return 2.0 * xp.exp(-1.0 * z) * xp.cos(x) * xp.sin(y)

    zero = lambda r: _xyz(r)[3].full(0.0)  # noqa: E731
    return _assemble(phi, u_m, u_p, mu_m, mu_p, zero, zero, f_m, f_p, beta)


def reference_star_problem():
    """``star()`` of tests/confs/experiment_configs.py:196-412: a three-mode star
    phi = |x| - r0 (1 + ((x^2+y^2)/|x|^2)^2 core(atan2(y, x))), u- = sin 2x cos 2y e^z,
    u+ = (16 t^5 - 20 t^3 + 5 t) ln(x + y + 3) cos z with t = (y - x)/3,
    mu- = 10 (1 + 0.2 cos 2pi(x+y) sin 2pi(x-y) cos z), mu+ = 1, k = 0, g = u+, f from the
    hand-written f_m_fn/f_p_fn (:355-397), beta = nan_to_num(-(mu+ grad u+ - mu- grad u-) . grad phi)
    with the unnormalised grad phi (:280-292).  mu- > mu+ everywhere (mu- >= 8)."""
    r0 = 0.483
    modes = ((3.0, 0.1, 0.5), (4.0, -0.1, 1.8), (7.0, 0.15, 0.0))

    def _core(r):
        x, y, z, xp = _xyz(r)
        th = xp.arctan2(y, x)
        c = 0.0
        dc = 0.0
        for n_i, b_i, t_i in modes:
            c = c + b_i * xp.cos(n_i * (th - t_i))
            dc = dc - b_i * n_i * xp.sin(n_i * (th - t_i))
        return c, dc

    def phi(r):
        x, y, z, xp = _xyz(r)
        s = x * x + y * y
        rho2 = s + z * z
        c, _ = _core(r)
        q = s / rho2  # 0/0 = NaN at the origin, where nan_to_num gives 0 (experiment_configs.py:248)
        v = xp.sqrt(rho2) - r0 * (1.0 + q * q * c)
        return xp.nan_to_num(v)

    def grad_phi(r):
        x, y, z, xp = _xyz(r)
        s = x * x + y * y
        rho2 = s + z * z
        rho = xp.sqrt(rho2)
        c, dc = _core(r)
        q = xp.safe_div(s, rho2)
        rho4 = rho2 * rho2
        dq = (xp.safe_div(2.0 * x * z * z, rho4), xp.safe_div(2.0 * y * z * z, rho4), xp.safe_div(-2.0 * s * z, rho4))
        dth = (xp.safe_div(-y, s), xp.safe_div(x, s), 0.0)
        out = []
        for a, u in enumerate((x, y, z)):
            out.append(xp.safe_div(u, rho) - r0 * (2.0 * q * dq[a] * c + q * q * dc * dth[a]))
        return out

    def u_m(r):
        x, y, z, xp = _xyz(r)
        return xp.sin(2.0 * x) * xp.cos(2.0 * y) * xp.exp(z)

    def _poly(t):
        return 16.0 * t ** 5 - 20.0 * t ** 3 + 5.0 * t

    def u_p(r):
        x, y, z, xp = _xyz(r)
        return _poly((y - x) / 3.0) * xp.log(x + y + 3.0) * xp.cos(z)

    def mu_m(r):
        x, y, z, xp = _xyz(r)
        pi = math.pi
        return 10.0 * (1.0 + 0.2 * xp.cos(2.0 * pi * (x + y)) * xp.sin(2.0 * pi * (x - y)) * xp.cos(z))

    def mu_p(r):
        return _xyz(r)[3].full(1.0)

    def f_m(r):
        x, y, z, xp = _xyz(r)
        pi = math.pi
        e = xp.exp(z)
        return (-1.0 * mu_m(r) * (-7.0 * xp.sin(2.0 * x) * xp.cos(2.0 * y) * e)
                + -4.0 * pi * xp.cos(z) * xp.cos(4.0 * pi * x) * 2.0 * xp.cos(2.0 * x) * xp.cos(2.0 * y) * e
                + -4.0 * pi * xp.cos(z) * xp.cos(4.0 * pi * y) * (-2.0) * xp.sin(2.0 * x) * xp.sin(2.0 * y) * e
                + 2.0 * xp.cos(2.0 * pi * (x + y)) * xp.sin(2.0 * pi * (x - y)) * xp.sin(z) * xp.sin(2.0 * x)
                * xp.cos(2.0 * y) * e)

    def f_p(r):
        x, y, z, xp = _xyz(r)
        t = (y - x) / 3.0
        L = xp.log(x + y + 3.0)
        cz = xp.cos(z)
        return -1.0 * (_poly(t) * (-2.0) * cz / (x + y + 3.0) ** 2
                       + 2.0 * (16.0 * 5.0 * 4.0 * (1.0 / 9.0) * t ** 3 - 20.0 * 3.0 * 2.0 * (1.0 / 9.0) * t) * L * cz
                       + -1.0 * _poly(t) * L * cz)

    def beta(r):
        x, y, z, xp = _xyz(r)
        gx, gy, gz = grad_phi(r)
        t = (y - x) / 3.0
        P = _poly(t)
        dP = (80.0 * t ** 4 - 60.0 * t ** 2 + 5.0) / 3.0  # d/dy; d/dx = -dP
        L = xp.log(x + y + 3.0)
        s3 = x + y + 3.0
        cz, sz = xp.cos(z), xp.sin(z)
        gup = (-dP * L * cz + P * cz / s3, dP * L * cz + P * cz / s3, -P * L * sz)
        e = xp.exp(z)
        s2x, c2x, s2y, c2y = xp.sin(2.0 * x), xp.cos(2.0 * x), xp.sin(2.0 * y), xp.cos(2.0 * y)
        gum = (2.0 * c2x * c2y * e, -2.0 * s2x * s2y * e, s2x * c2y * e)
        mp, mm = 1.0, mu_m(r)
        d = (mp * gup[0] - mm * gum[0]) * gx + (mp * gup[1] - mm * gum[1]) * gy + (mp * gup[2] - mm * gum[2]) * gz
        return xp.nan_to_num(d * (-1.0))

    zero = lambda r: _xyz(r)[3].full(0.0)  # noqa: E731
    return _assemble(phi, u_m, u_p, mu_m, mu_p, zero, zero, f_m, f_p, beta)


def _assemble(phi, u_m, u_p, mu_m, mu_p, k_m, k_p, f_m, f_p, beta):
    def alpha(r):
        return u_p(r) - u_m(r)

    def exact(r):
        x, y, z, xp = _xyz(r)
        return xp.where(phi(r) >= 0, u_p(r), u_m(r))

    return {
        "phi": phi,
        "mu_m": mu_m,
        "mu_p": mu_p,
        "k_m": k_m,
        "k_p": k_p,
        "f_m": f_m,
        "f_p": f_p,
        "alpha": alpha,
        "beta": beta,
        "g": u_p,
        "u_m": u_m,
        "u_p": u_p,
        "exact": exact,
    }


# ----------------------------------------------------------------------------------------
# irregular blob (config 5): phi = 0.3 - sum of 500 Gaussians
# ----------------------------------------------------------------------------------------
def blob_problem(n_gauss=500, seed=0, iso=0.3, mu_m=1.0, mu_p=100.0, k=0.5):
    """phi = iso - sum_i exp(-|x - c_i|^2 / (2 w_i^2)), centres uniform in [-0.7, 0.7]^3, widths
    uniform in [0.05, 0.2] (numpy default_rng(seed)); mu- = 1, mu+ = 100, k+- = 0.5;
    u- = sin x cos y e^z, u+ = x^2 + y^2 + z^2 (the sphere problem's solution)."""
    rng = np.random.default_rng(seed)
    C = rng.uniform(-0.7, 0.7, (n_gauss, 3)).astype(np.float32)
    Wd = rng.uniform(0.05, 0.2, n_gauss).astype(np.float32)
    inv2w2 = (1.0 / (2.0 * Wd.astype(np.float64) ** 2)).astype(np.float32)
    invw2 = (1.0 / Wd.astype(np.float64) ** 2).astype(np.float32)
    cache = {}

    def _tables(r):
        if _is_torch(r):
            key = str(r.device)
            if key not in cache:
                cache[key] = tuple(torch.as_tensor(a, device=r.device) for a in (C, inv2w2, invw2))
            return cache[key]
        return C, inv2w2, invw2

    def _sum(r, want_grad):
        """S(x) and (optionally) grad S, points in chunks and Gaussians in blocks of 32."""
        c, a, b = _tables(r[0])
        xp = _NS(r[0])
        M = r[0].shape[0]
        S = xp.full(0.0)
        G = [xp.full(0.0), xp.full(0.0), xp.full(0.0)] if want_grad else None
        step = 1 << 19
        for p0 in range(0, M, step):
            p1 = min(M, p0 + step)
            x, y, z = r[0][p0:p1, None], r[1][p0:p1, None], r[2][p0:p1, None]
            for g0 in range(0, c.shape[0], 32):
                g1 = min(c.shape[0], g0 + 32)
                dx, dy, dz = x - c[g0:g1, 0], y - c[g0:g1, 1], z - c[g0:g1, 2]
                e = xp.exp(-(dx * dx + dy * dy + dz * dz) * a[g0:g1])
                S[p0:p1] += e.sum(1)
                if want_grad:
                    eb = e * b[g0:g1]
                    G[0][p0:p1] -= (eb * dx).sum(1)
                    G[1][p0:p1] -= (eb * dy).sum(1)
                    G[2][p0:p1] -= (eb * dz).sum(1)
        return S, G

    def phi(r):
        S, _ = _sum(r, False)
        return iso - S

    def u_m(r):
        x, y, z, xp = _xyz(r)
        return xp.sin(x) * xp.cos(y) * xp.exp(z)

    def u_p(r):
        x, y, z, xp = _xyz(r)
        return x * x + y * y + z * z

    def f_m(r):  # -mu- lap u- + k u-, lap u- = -u-
        return (mu_m + k) * u_m(r)

    def f_p(r):  # -mu+ lap u+ + k u+, lap u+ = 6
        return -6.0 * mu_p + k * u_p(r)

    def beta(r):
        x, y, z, xp = _xyz(r)
        _, gS = _sum(r, True)
        gx, gy, gz = -gS[0], -gS[1], -gS[2]  # grad phi = -grad S
        gn = xp.sqrt(gx * gx + gy * gy + gz * gz)
        nx, ny, nz = xp.safe_div(gx, gn), xp.safe_div(gy, gn), xp.safe_div(gz, gn)
        e = xp.exp(z)
        dn_um = xp.cos(x) * xp.cos(y) * e * nx - xp.sin(x) * xp.sin(y) * e * ny + xp.sin(x) * xp.cos(y) * e * nz
        dn_up = 2.0 * (x * nx + y * ny + z * nz)
        return -(mu_p * dn_up - mu_m * dn_um)

    return _assemble(phi, u_m, u_p, lambda r: _xyz(r)[3].full(mu_m), lambda r: _xyz(r)[3].full(mu_p),
                     lambda r: _xyz(r)[3].full(k), lambda r: _xyz(r)[3].full(k), f_m, f_p, beta)


# ----------------------------------------------------------------------------------------
# linearised Poisson-Boltzmann instances (config 4)
# ----------------------------------------------------------------------------------------
def lpbe_problem(centres, radii, charges, sigma=0.02, mu_m=1.0, mu_p=80.0, k_p=0.1):
    """phi = min_i(|x - c_i| - r_i); f- = sum_i q_i N(c_i, sigma); zero Dirichlet BC, no jumps.

    The form follows examples/benchmark_LPBE/geometry.py:20-37 and coefficients.py:266-291.
    """
    C = np.asarray(centres, np.float32)
    R = np.asarray(radii, np.float32)
    Q = np.asarray(charges, np.float32)
    norm = 1.0 / ((2.0 * math.pi) ** 1.5 * sigma ** 3)

    def _cols(r):
        if _is_torch(r):
            dev = r.device
            return (torch.as_tensor(C, device=dev), torch.as_tensor(R, device=dev), torch.as_tensor(Q, device=dev))
        return C, R, Q

    def phi(r):
        c, rad, _ = _cols(r)
        xp = _NS(r[0])
        out = None
        for i in range(c.shape[0]):
            d = xp.sqrt((r[0] - c[i, 0]) ** 2 + (r[1] - c[i, 1]) ** 2 + (r[2] - c[i, 2]) ** 2) - rad[i]
            out = d if out is None else xp.minimum(out, d)
        return out

    def f_m(r):
        c, _, q = _cols(r)
        xp = _NS(r[0])
        out = xp.full(0.0)
        for i in range(c.shape[0]):
            if float(q[i]) == 0.0:
                continue
            d2 = (r[0] - c[i, 0]) ** 2 + (r[1] - c[i, 1]) ** 2 + (r[2] - c[i, 2]) ** 2
            out = out + q[i] * norm * xp.exp(-d2 / (2.0 * sigma * sigma))
        return out

    zero = lambda r: _NS(r[0]).full(0.0)  # noqa: E731
    return {
        "phi": phi,
        "mu_m": lambda r: _NS(r[0]).full(mu_m),
        "mu_p": lambda r: _NS(r[0]).full(mu_p),
        "k_m": zero,
        "k_p": lambda r: _NS(r[0]).full(k_p),
        "f_m": f_m,
        "f_p": zero,
        "alpha": zero,
        "beta": zero,
        "g": zero,
    }


def lpbe_instances(n_instances=64, seed=0):
    """Seeded synthetic stand-ins for the 64 uneven LPBE instances (sides 48..160 step 16)."""
    rng = np.random.default_rng(seed)
    out = []
    sides = np.arange(48, 161, 16)
    for _ in range(n_instances):
        side = int(rng.choice(sides))
        ns = int(rng.integers(50, 2001))
        c = rng.uniform(-0.6, 0.6, (ns, 3)).astype(np.float32)
        r = rng.uniform(0.05, 0.12, ns).astype(np.float32)
        q = rng.integers(-1, 2, ns).astype(np.float32)
        out.append((side, c, r, q))
    return out


def exact_solution(prob, pts):
    """u_exact at points (N,3) (numpy)."""
    return np.asarray(prob["exact"](np.asarray(pts, np.float32).T), np.float32)
