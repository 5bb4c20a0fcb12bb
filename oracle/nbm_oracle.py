"""CPU oracle for the NBM jump-condition finite-volume residual.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
do, and only to check results (or as the timed CPU restatement of the reference).

This file restates, in numpy float32, the reference's geometry and
interpolation for the per-point FV residual (JAX-DIPS 0.2.1, x64 disabled):

* grids        -- ``jax.numpy.linspace`` (jax 0.4.13) and ``domain/mesh.py:121-153``
* level set    -- ``geometry/level_set.py:34-48`` (perturbation)
* trilinear phi-- ``domain/interpolate.py:762-816`` (ghost layer) and ``:906-1021``
* cell geometry-- ``geometry/geometric_integrations_per_point.py:32-1009``
* regression   -- ``solvers/poisson/discretization.py:164-296``
* batching     -- ``data/data_management.py:79-159, 319-326``
* optimizer    -- ``solvers/optimizers.py:13-54`` (optax 0.1.5 semantics)

Every function is vectorised over points the way the reference ``vmap``s its
per-point functions; each keeps the reference's evaluation order of float32
operations wherever a discrete decision (sign tests, ``isclose`` face tests,
stable argsorts) depends on the rounded value.

PARITY STATUS: parity unpinned.  jax/jaxlib/haiku/optax are not installable
here, so the reference cannot be run to produce golden vectors, and the
reference's own tests hold no golden residual, loss or gradient values.  The
only known-answer test on this path is the geometric-integration test
(``tests/test_geometric_integrations.py:172-182``: interface area of the
r=0.5 sphere = pi +- 0.02, enclosed volume = pi/6 +- 0.02 on a 128^3 grid over
[-2,2]^3); this oracle is pinned against it (tests/test_oracle.py).

Two places where the restatement differs from jax arithmetic on purpose, both
continuous (no discrete decision depends on them):

* ``jnp.linalg.pinv`` (fp32 SVD, cutoff 10*max(m,n)*eps*sigma_max) is
  evaluated in float64 with the same cutoff rule; the rank decision is robust
  because X^T W X = S M S with M an integer matrix.
* ``jnp.linalg.det`` uses jax's closed-form 2x2/3x3 expressions.
"""

from __future__ import annotations

import numpy as np

F32 = np.float32
I32 = np.int32


# ----------------------------------------------------------------------------------------
# grids
# ----------------------------------------------------------------------------------------
def linspace_f32(start, stop, num):
    """``jnp.linspace(start, stop, num, dtype=f32)`` with x64 off.

    jax computes ``start*(1-t) + stop*t`` with ``t = iota/(num-1)`` in float32
    and appends ``stop`` exactly.
    """
    start = F32(start)
    stop = F32(stop)
    if num == 1:
        return np.array([start], F32)
    div = num - 1
    t = (np.arange(div, dtype=F32) / F32(div)).astype(F32)
    out = (start * (F32(1.0) - t) + stop * t).astype(F32)
    return np.concatenate([out, np.array([stop], F32)]).astype(F32)


def grid_points(x, y, z):
    """``mesh.construct(3)`` point ordering: meshgrid 'ij', C-order flatten (mesh.py:125-129)."""
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(F32)


def grid_spacing(x):
    """``dx = x[1] - x[0]`` (mesh.py:122)."""
    return F32(x[1] - x[0])


# ----------------------------------------------------------------------------------------
# level set
# ----------------------------------------------------------------------------------------
def perturb(phi):
    """``perturb_level_set_fn`` (level_set.py:34-48): phi + sign_pm(phi)*1e-10, phi=0 -> -1e-10."""
    phi = np.asarray(phi, F32)
    sgn = np.sign(np.sign(phi) - F32(0.5)).astype(F32)
    return (phi + sgn * F32(1.0e-10)).astype(F32)


def ghost_layer_3d(c):
    """``add_ghost_layer_3d`` (interpolate.py:762-816): linear extrapolation 2*c0 - c1, x then y then z."""
    c = np.asarray(c, F32)
    nx, ny, nz = c.shape
    g = np.zeros((nx + 2, ny + 2, nz + 2), F32)
    g[1:-1, 1:-1, 1:-1] = c
    two = F32(2.0)
    g[0, 1:-1, 1:-1] = two * c[0] - c[1]
    g[-1, 1:-1, 1:-1] = two * c[-1] - c[-2]
    yb = two * g[:, 1, :] - g[:, 2, :]
    yt = two * g[:, -2, :] - g[:, -3, :]
    g[:, 0, :] = yb
    g[:, -1, :] = yt
    zb = two * g[:, :, 1] - g[:, :, 2]
    zt = two * g[:, :, -2] - g[:, :, -3]
    g[:, :, 0] = zb
    g[:, :, -1] = zt
    return g


def ghost_coords(x):
    x = np.asarray(x, F32)
    xx = np.zeros(x.shape[0] + 2, F32)
    xx[1:-1] = x
    xx[0] = x[0] - (x[1] - x[0])
    xx[-1] = x[-1] + (x[-1] - x[-2])
    return xx


class Trilinear:
    """``multilinear_interpolation(c, gstate)`` (interpolate.py:906-1021), float32.

    The lower-left ghosted index ``i32((x-x0)/dx)`` is clamped to [2, n-2]; the
    first real cell is therefore extrapolated from the next one (reference quirk).
    """

    def __init__(self, values, x, y, z):
        x = np.asarray(x, F32)
        y = np.asarray(y, F32)
        z = np.asarray(z, F32)
        cube = np.asarray(values, F32).reshape(x.shape[0], y.shape[0], z.shape[0])
        self.gh = ghost_layer_3d(cube)
        self.xx, self.yy, self.zz = ghost_coords(x), ghost_coords(y), ghost_coords(z)

    @staticmethod
    def _index(p, axis):
        n = axis.shape[0]
        d = axis[1] - axis[0]
        with np.errstate(invalid="ignore"):
            q = (p - axis[0]) / d
            q = np.where(np.isfinite(q), q, 0.0)
            q = np.clip(q, -2.0**31, 2.0**31 - 128)
        i = q.astype(I32)  # truncation toward zero, as int32 conversion
        i = np.where(i >= n - 1, I32(n - 2), i)
        i = np.where(i <= 1, I32(2), i)
        return i

    def __call__(self, pts):
        pts = np.asarray(pts, F32)
        shp = pts.shape[:-1]
        pts = pts.reshape(-1, 3)
        xp, yp, zp = pts[:, 0], pts[:, 1], pts[:, 2]
        xx, yy, zz, g = self.xx, self.yy, self.zz, self.gh
        i = self._index(xp, xx)
        j = self._index(yp, yy)
        k = self._index(zp, zz)
        c111 = g[i + 1, j + 1, k + 1]
        c110 = g[i + 1, j + 1, k]
        c011 = g[i, j + 1, k + 1]
        c101 = g[i + 1, j, k + 1]
        c001 = g[i, j, k + 1]
        c010 = g[i, j + 1, k]
        c100 = g[i + 1, j, k]
        c000 = g[i, j, k]
        one = F32(1.0)
        xd = (xp - xx[i]) / (xx[i + 1] - xx[i])
        yd = (yp - yy[j]) / (yy[j + 1] - yy[j])
        zd = (zp - zz[k]) / (zz[k + 1] - zz[k])
        c00 = c000 * (one - xd) + c100 * xd
        c01 = c001 * (one - xd) + c101 * xd
        c10 = c010 * (one - xd) + c110 * xd
        c11 = c011 * (one - xd) + c111 * xd
        c0 = c00 * (one - yd) + c10 * yd
        c1 = c01 * (one - yd) + c11 * yd
        c = c0 * (one - zd) + c1 * zd
        return c.astype(F32).reshape(shp)

    def quadratic(self, pts):
        """``nonoscillatory_quadratic_interpolation`` (interpolate.py:572-759), float32: the
        trilinear value minus 0.5 t (1 - t) min|second difference| per axis over the cell's 8
        corners; out-of-range neighbour indices clamp into the ghosted cube (jax gathers clamp)."""
        pts = np.asarray(pts, F32)
        shp = pts.shape[:-1]
        pts = pts.reshape(-1, 3)
        xp, yp, zp = pts[:, 0], pts[:, 1], pts[:, 2]
        xx, yy, zz, g = self.xx, self.yy, self.zz, self.gh
        n0, n1, n2 = g.shape
        i = self._index(xp, xx)
        j = self._index(yp, yy)
        k = self._index(zp, zz)

        def at(a, b, c):
            return g[np.clip(a, 0, n0 - 1), np.clip(b, 0, n1 - 1), np.clip(c, 0, n2 - 1)]

        two, half, one = F32(2.0), F32(0.5), F32(1.0)
        mins = []
        for di, dj, dk in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
            m = None
            for a in (0, 1):
                for b in (0, 1):
                    for c in (0, 1):
                        I, J, K = i + a, j + b, k + c
                        d2 = (at(I + di, J + dj, K + dk) - two * at(I, J, K)) + at(I - di, J - dj, K - dk)
                        m = np.abs(d2) if m is None else np.minimum(m, np.abs(d2))
            mins.append(m)
        xd = (xp - xx[i]) / (xx[i + 1] - xx[i])
        yd = (yp - yy[j]) / (yy[j + 1] - yy[j])
        zd = (zp - zz[k]) / (zz[k + 1] - zz[k])
        v = self(pts).reshape(-1)
        v = v - mins[0] * half * xd * (one - xd)
        v = v - mins[1] * half * yd * (one - yd)
        v = v - mins[2] * half * zd * (one - zd)
        return v.astype(F32).reshape(shp)


# ----------------------------------------------------------------------------------------
# small fp32 helpers restating jnp semantics
# ----------------------------------------------------------------------------------------
def sign_m(a):
    """1 where a < 0 else 0 (geom_pp.py:45-49)."""
    return (np.asarray(a) < 0).astype(F32)


def sign_p(a):
    """1 where a > 0 else 0 (geom_pp.py:38-42)."""
    return (np.asarray(a) > 0).astype(F32)


def nan_to_num(a):
    a = np.asarray(a, F32)
    return np.nan_to_num(a, nan=F32(0.0), posinf=np.finfo(F32).max, neginf=np.finfo(F32).min).astype(F32)


def isclose_f32(a, b, atol):
    """``jnp.isclose(a, b, atol=atol)`` (rtol=1e-5) in float32."""
    a = np.asarray(a, F32)
    b = np.asarray(b, F32)
    with np.errstate(invalid="ignore"):
        out = np.abs(a - b) <= (F32(atol) + F32(1e-5) * np.abs(b))
        out &= ~(np.isinf(a) | np.isinf(b))
        out |= np.isinf(a) & np.isinf(b) & (a == b)
        out &= ~(np.isnan(a) | np.isnan(b))
    return out


def _dot3(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def _det2(g):
    return g[..., 0, 0] * g[..., 1, 1] - g[..., 0, 1] * g[..., 1, 0]


def _det3(a):
    return (
        a[..., 0, 0] * a[..., 1, 1] * a[..., 2, 2]
        + a[..., 0, 1] * a[..., 1, 2] * a[..., 2, 0]
        + a[..., 0, 2] * a[..., 1, 0] * a[..., 2, 1]
        - a[..., 0, 2] * a[..., 1, 1] * a[..., 2, 0]
        - a[..., 0, 0] * a[..., 1, 2] * a[..., 2, 1]
        - a[..., 0, 1] * a[..., 1, 0] * a[..., 2, 2]
    )


def area_fn(tri):
    """``area_fn`` (geom_pp.py:377-380, :502-507): 0.5*sqrt|det(D D^T)|, D = A[1:] - A[0]."""
    tri = np.asarray(tri, F32)
    d = tri[..., 1:, :] - tri[..., :1, :]
    g = np.empty(d.shape[:-2] + (2, 2), F32)
    for a in range(2):
        for b in range(2):
            g[..., a, b] = _dot3(d[..., a, :], d[..., b, :])
    with np.errstate(invalid="ignore", over="ignore"):
        return (F32(0.5) * np.sqrt(np.abs(nan_to_num(_det2(g))))).astype(F32)


def vol_fn(tet):
    """``vol_fn`` (geom_pp.py:370-374, :496-500): (1/6)*sqrt|det(D D^T)|."""
    tet = np.asarray(tet, F32)
    d = tet[..., 1:, :] - tet[..., :1, :]
    g = np.empty(d.shape[:-2] + (3, 3), F32)
    for a in range(3):
        for b in range(3):
            g[..., a, b] = _dot3(d[..., a, :], d[..., b, :])
    with np.errstate(invalid="ignore", over="ignore"):
        return (F32(1.0 / 6.0) * np.sqrt(np.abs(nan_to_num(_det3(g))))).astype(F32)


# ----------------------------------------------------------------------------------------
# cell geometry (geometric_integrations_per_point.py)
# ----------------------------------------------------------------------------------------
# corner offsets P_000, P_100, P_101, P_001, P_010, P_110, P_011, P_111 (geom_pp.py:214-226)
CORNER_SIGNS = np.array(
    [[-1, -1, -1], [1, -1, -1], [1, -1, 1], [-1, -1, 1], [-1, 1, -1], [1, 1, -1], [-1, 1, 1], [1, 1, 1]],
    dtype=np.int64,
)
# five-tetrahedron split S1..S5 as corner indices (geom_pp.py:311-322)
TETS = np.array([[0, 1, 4, 3], [5, 1, 4, 7], [2, 1, 7, 3], [6, 7, 4, 3], [7, 1, 4, 3]], dtype=np.int64)


def corner_offsets(h):
    h = np.asarray(h, F32)
    return (CORNER_SIGNS.astype(F32) * h[None, :]).astype(F32) * F32(0.5)


def cell_corners(p, h):
    return (np.asarray(p, F32)[:, None, :] + corner_offsets(h)[None]).astype(F32)


def crossed_from_corner_phi(phic):
    """``is_point_cell_crossed_by_interface`` (geom_pp.py:203-263): +-1 if all 8 share a sign else 0."""
    eta = (phic < 0).sum(axis=1)
    s0 = np.sign(phic[:, 0]).astype(F32)
    return np.where((eta == 0) | (eta == 8), s0, F32(0.0)).astype(F32)


def is_crossed(phi_fn, p, h):
    corners = cell_corners(p, h)
    phic = phi_fn(corners.reshape(-1, 3)).reshape(-1, 8)
    return crossed_from_corner_phi(phic)


def _sorted(S, ph):
    order = np.argsort(ph, axis=1, kind="stable")
    Ss = np.take_along_axis(S, order[:, :, None], axis=1)
    ps = np.take_along_axis(ph, order, axis=1)
    return Ss, ps


def _lerp(Ss, ps, i, j):
    """(phi_i*S_j - phi_j*S_i)/(phi_i - phi_j), componentwise in float32."""
    with np.errstate(divide="ignore", invalid="ignore"):
        num = ps[:, i, None] * Ss[:, j, :] - ps[:, j, None] * Ss[:, i, :]
        den = ps[:, i, None] - ps[:, j, None]
        return (num / den).astype(F32)


def tet_gamma(S, ph, eta):
    """``get_vertices_S_intersect_Gamma`` (geom_pp.py:52-107) -> (N, 2, 3, 3)."""
    N = S.shape[0]
    out = np.zeros((N, 2, 3, 3), F32)
    Ss, ps = _sorted(S, ph)
    e1 = np.stack([_lerp(Ss, ps, 0, 1), _lerp(Ss, ps, 0, 2), _lerp(Ss, ps, 0, 3)], axis=1)
    q0, q1, q2, q5 = _lerp(Ss, ps, 0, 2), _lerp(Ss, ps, 0, 3), _lerp(Ss, ps, 1, 3), _lerp(Ss, ps, 1, 2)
    e2a = np.stack([q0, q1, q2], axis=1)
    e2b = np.stack([q0, q5, q2], axis=1)
    Sn, pn = _sorted(S, -ph)
    e3 = np.stack([_lerp(Sn, pn, 0, 1), _lerp(Sn, pn, 0, 2), _lerp(Sn, pn, 0, 3)], axis=1)
    m1 = eta == 1
    m2 = eta == 2
    m3 = eta == 3
    out[m1, 0] = e1[m1]
    out[m2, 0] = e2a[m2]
    out[m2, 1] = e2b[m2]
    out[m3, 0] = e3[m3]
    return out


def tet_omega_m(S, ph, eta):
    """``get_vertices_S_intersect_Omega_m`` (geom_pp.py:110-198) -> (N, 3, 4, 3)."""
    N = S.shape[0]
    out = np.zeros((N, 3, 4, 3), F32)
    Ss, ps = _sorted(S, ph)
    L = lambda i, j: _lerp(Ss, ps, i, j)  # noqa: E731
    e1 = np.stack([Ss[:, 0], L(0, 1), L(0, 2), L(0, 3)], axis=1)
    Q0, Q1 = Ss[:, 0], Ss[:, 1]
    Q2, Q3, Q4, Q5 = L(0, 2), L(1, 3), L(1, 2), L(0, 3)
    e2 = np.stack(
        [np.stack([Q0, Q1, Q2, Q3], 1), np.stack([Q4, Q1, Q2, Q3], 1), np.stack([Q0, Q5, Q2, Q3], 1)], axis=1
    )
    R0, R1, R2 = Ss[:, 0], Ss[:, 1], Ss[:, 2]
    R3, R4, R5 = L(1, 3), L(0, 3), L(2, 3)
    e3 = np.stack(
        [np.stack([R0, R1, R2, R3], 1), np.stack([R0, R4, R2, R3], 1), np.stack([R5, R4, R2, R3], 1)], axis=1
    )
    m1, m2, m3, m4 = eta == 1, eta == 2, eta == 3, eta == 4
    out[m1, 0] = e1[m1]
    out[m2] = e2[m2]
    out[m3] = e3[m3]
    out[m4, 0] = S[m4]
    return out


class CellGeometry:
    """Five-tet decomposition of the h-cube centred at each point (geom_pp.py:266-362)."""

    def __init__(self, phi_fn, p, h):
        self.p = np.asarray(p, F32)
        self.h = np.asarray(h, F32)
        N = self.p.shape[0]
        self.corners = cell_corners(self.p, self.h)
        self.phic = phi_fn(self.corners.reshape(-1, 3)).reshape(N, 8).astype(F32)
        self.crossed = crossed_from_corner_phi(self.phic)
        self.gamma = []
        self.omega = []
        for t in TETS:
            S = self.corners[:, t]
            ph = self.phic[:, t]
            eta = (ph < 0).sum(axis=1)
            self.gamma.append(tet_gamma(S, ph, eta))
            self.omega.append(tet_omega_m(S, ph, eta))


def _face_partition_area(part, on_face):
    """``compute_area_from_partitions.comp`` (geom_pp.py:584-626) for one (N,3,4,3) partition."""
    fid = F32(200.0)
    P = np.where(on_face[..., None], part, fid).astype(F32)
    num = np.count_nonzero(P[..., 0] - fid, axis=-1)
    order = np.argsort(P[..., 0], axis=-1, kind="stable")
    Ps = np.take_along_axis(P, order[..., None], axis=2)[:, :, :3, :]
    a = area_fn(Ps)
    a = np.where(num == 3, a, F32(0.0)).astype(F32)
    return ((a[:, 0] + a[:, 1]) + a[:, 2]).astype(F32)


def face_area_m(om_a, om_b, axis, face_coord, h_axis):
    """``extract_area_minus_{x,y,z}_face`` (geom_pp.py:811-839)."""
    atol = F32(1e-10) * F32(h_axis)
    fa = isclose_f32(om_a[..., axis], face_coord[:, None, None], atol)
    fb = isclose_f32(om_b[..., axis], face_coord[:, None, None], atol)
    return (_face_partition_area(om_a, fa) + _face_partition_area(om_b, fb)).astype(F32)


def face_centres(p, h):
    """Face centres of the h-cube (geom_pp.py:533-545): order imh, iph, jmh, jph, kmh, kph."""
    h = np.asarray(h, F32)
    d = np.zeros((6, 3), F32)
    d[0, 0], d[1, 0] = -h[0], h[0]
    d[2, 1], d[3, 1] = -h[1], h[1]
    d[4, 2], d[5, 2] = -h[2], h[2]
    d = F32(0.5) * d
    return (np.asarray(p, F32)[:, None, :] + d[None]).astype(F32)


def face_coefficients(geo: CellGeometry, mu_m_faces, mu_p_faces):
    """``compute_face_centroids_values_plus_minus_at_point`` (geom_pp.py:998-1007) -> (N, 26)."""
    p, h = geo.p, geo.h
    dx, dy, dz = h[0], h[1], h[2]
    N = p.shape[0]
    vol = dx * dy * dz
    area_x, area_y, area_z = dy * dz, dx * dz, dx * dy
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    half = F32(0.5)
    pz = lambda v: np.where(v < 0, F32(0.0), v).astype(F32)  # noqa: E731

    # ---- interface cells (geom_pp.py:514-903)
    vol_m = np.zeros(N, F32)
    first = True
    for t in range(5):
        for q in range(3):
            v = vol_fn(geo.omega[t][:, q])
            vol_m = v if first else (vol_m + v).astype(F32)
            first = False
    vol_p = pz(vol - vol_m)
    S1, S2, S3, S4 = geo.omega[0], geo.omega[1], geo.omega[2], geo.omega[3]
    a_imh_m = face_area_m(S1, S4, 0, x - half * dx, dx)
    a_iph_m = face_area_m(S2, S3, 0, x + half * dx, dx)
    a_jmh_m = face_area_m(S1, S3, 1, y - half * dy, dy)
    a_jph_m = face_area_m(S2, S4, 1, y + half * dy, dy)
    a_kmh_m = face_area_m(S1, S2, 2, z - half * dz, dz)
    a_kph_m = face_area_m(S3, S4, 2, z + half * dz, dz)
    a_imh_p, a_iph_p = pz(area_x - a_imh_m), pz(area_x - a_iph_m)
    a_jmh_p, a_jph_p = pz(area_y - a_jmh_m), pz(area_y - a_jph_m)
    a_kmh_p, a_kph_p = pz(area_z - a_kmh_m), pz(area_z - a_kph_m)
    mm, mp = np.asarray(mu_m_faces, F32), np.asarray(mu_p_faces, F32)
    itf = np.stack(
        [
            a_imh_m * mm[:, 0] / dx,
            a_imh_p * mp[:, 0] / dx,
            a_iph_m * mm[:, 1] / dx,
            a_iph_p * mp[:, 1] / dx,
            a_jmh_m * mm[:, 2] / dy,
            a_jmh_p * mp[:, 2] / dy,
            a_jph_m * mm[:, 3] / dy,
            a_jph_p * mp[:, 3] / dy,
            a_kmh_m * mm[:, 4] / dz,
            a_kmh_p * mp[:, 4] / dz,
            a_kph_m * mm[:, 5] / dz,
            a_kph_p * mp[:, 5] / dz,
            vol_m,
            vol_p,
            a_imh_m,
            a_imh_p,
            a_iph_m,
            a_iph_p,
            a_jmh_m,
            a_jmh_p,
            a_jph_m,
            a_jph_p,
            a_kmh_m,
            a_kmh_p,
            a_kph_m,
            a_kph_p,
        ],
        axis=1,
    ).astype(F32)

    # ---- domain cells (geom_pp.py:905-996)
    c = geo.crossed
    msk_m, msk_p = sign_m(c), sign_p(c)
    dm = mm * msk_m[:, None]
    dp = mp * msk_p[:, None]
    dom = np.stack(
        [
            area_x * dm[:, 0] / dx,
            area_x * dp[:, 0] / dx,
            area_x * dm[:, 1] / dx,
            area_x * dp[:, 1] / dx,
            area_y * dm[:, 2] / dy,
            area_y * dp[:, 2] / dy,
            area_y * dm[:, 3] / dy,
            area_y * dp[:, 3] / dy,
            area_z * dm[:, 4] / dz,
            area_z * dp[:, 4] / dz,
            area_z * dm[:, 5] / dz,
            area_z * dp[:, 5] / dz,
            vol * msk_m,
            vol * msk_p,
            area_x * msk_m,
            area_x * msk_p,
            area_x * msk_m,
            area_x * msk_p,
            area_y * msk_m,
            area_y * msk_p,
            area_y * msk_m,
            area_y * msk_p,
            area_z * msk_m,
            area_z * msk_p,
            area_z * msk_m,
            area_z * msk_p,
        ],
        axis=1,
    ).astype(F32)
    return np.where((c == 0)[:, None], itf, dom).astype(F32)


def interface_integral(geo: CellGeometry, f_fn):
    """``integrate_over_interface_at_point`` (geom_pp.py:383-420): sum of area*mean(f) over 10 triangles.

    Padding triangles (zero vertices) are evaluated too, exactly as the reference does.
    """
    N = geo.p.shape[0]
    integral = None
    for t in range(5):
        for q in range(2):
            tri = geo.gamma[t][:, q]
            a = area_fn(tri)
            fv = np.asarray(f_fn(tri.reshape(-1, 3)), F32).reshape(N, 3)
            mean = ((fv[:, 0] + fv[:, 1]) + fv[:, 2]) / F32(3.0)
            term = (a * mean).astype(F32)
            integral = term if integral is None else (integral + term).astype(F32)
    return np.where(geo.crossed == 0, integral, F32(0.0)).astype(F32)


def negative_volume_integral(geo: CellGeometry, f_fn):
    """``integrate_in_negative_domain_at_point`` (geom_pp.py:422-459)."""
    N = geo.p.shape[0]
    integral = None
    for t in range(5):
        for q in range(3):
            tet = geo.omega[t][:, q]
            v = vol_fn(tet)
            fv = np.asarray(f_fn(tet.reshape(-1, 3)), F32).reshape(N, 4)
            mean = (((fv[:, 0] + fv[:, 1]) + fv[:, 2]) + fv[:, 3]) / F32(4.0)
            term = (v * mean).astype(F32)
            integral = term if integral is None else (integral + term).astype(F32)
    return integral


# ----------------------------------------------------------------------------------------
# least-squares regression of the jump extrapolation (discretization.py:164-296)
# ----------------------------------------------------------------------------------------
def xijk(h):
    """27 cube offsets, x fastest then y then z (discretization.py:164-197)."""
    h = np.asarray(h, F32)
    o = np.array([[ix, iy, iz] for iz in (-1, 0, 1) for iy in (-1, 0, 1) for ix in (-1, 0, 1)], np.int64)
    X = np.zeros((27, 3), F32)
    for c in range(3):
        X[:, c] = np.where(o[:, c] < 0, -h[c], np.where(o[:, c] > 0, h[c], F32(0.0)))
    return X


def pinv_lsq(X, w):
    """pinv(X^T W X) (W X)^T for each row of weights ``w`` (N, 27) -> (N, 3, 27) float32.

    Evaluated in float64 with jax's pinv cutoff (10*max(m,n)*eps_f32 * sigma_max).
    """
    X64 = X.astype(np.float64)
    w64 = w.astype(np.float64)
    WX = w64[:, :, None] * X64[None]  # (N,27,3)
    M = np.einsum("ki,nkj->nij", X64, WX)  # X^T W X
    u, s, vt = np.linalg.svd(M)
    cutoff = 10.0 * 3 * np.finfo(np.float32).eps * s[:, :1]
    sinv = np.where(s > cutoff, 1.0 / np.where(s > cutoff, s, 1.0), 0.0)
    pinv = np.einsum("nji,nj,nkj->nik", vt, sinv, u)
    D = np.einsum("nij,nkj->nik", pinv, WX)
    return np.nan_to_num(D.astype(F32))


class Regression:
    """``get_regression_coeffs_at_point`` (discretization.py:238-296) at stencil points s."""

    def __init__(self, phi_fn, s, h, mu_m_s, mu_p_s):
        s = np.asarray(s, F32)
        h = np.asarray(h, F32)
        N = s.shape[0]
        X = xijk(h)
        self.vertices = (s[:, None, :] + X[None]).astype(F32)  # (N,27,3)
        self.phi_vertices = phi_fn(self.vertices.reshape(-1, 3)).reshape(N, 27).astype(F32)
        Dp = pinv_lsq(X, sign_p(self.phi_vertices))
        Dm = pinv_lsq(X, sign_m(self.phi_vertices))
        dx, dy, dz = h
        two = F32(2.0)

        def shifted(c, d):
            q = s.copy()
            q[:, c] = s[:, c] + d
            return q

        phx = (phi_fn(shifted(0, dx)) - phi_fn(shifted(0, -dx))) / (two * dx)
        phy = (phi_fn(shifted(1, dy)) - phi_fn(shifted(1, -dy))) / (two * dy)
        phz = (phi_fn(shifted(2, dz)) - phi_fn(shifted(2, -dz))) / (two * dz)
        with np.errstate(divide="ignore", invalid="ignore"):
            norm = np.sqrt((phx * phx + phy * phy) + phz * phz)
            n = np.stack([phx / norm, phy / norm, phz / norm], axis=1).astype(F32)
        self.normal = n
        self.phi = phi_fn(s).astype(F32)
        Cm = ((n[:, 0, None] * Dm[:, 0] + n[:, 1, None] * Dm[:, 1]) + n[:, 2, None] * Dm[:, 2]).astype(F32)
        Cp = ((n[:, 0, None] * Dp[:, 0] + n[:, 1, None] * Dp[:, 1]) + n[:, 2, None] * Dp[:, 2]).astype(F32)
        mm = np.asarray(mu_m_s, F32)
        mp = np.asarray(mu_p_s, F32)
        with np.errstate(divide="ignore", invalid="ignore"):
            zp_pqm = (((mp - mm) / mm) * self.phi)[:, None] * Cp
            zm_pqm = (((mp - mm) / mp) * self.phi)[:, None] * Cm
            zp = -(zp_pqm.sum(axis=1, dtype=F32) - zp_pqm[:, 13])
            zm = -(zm_pqm.sum(axis=1, dtype=F32) - zm_pqm[:, 13])
            gp_pqm = zp_pqm / (F32(1.0) + zp)[:, None]
            gm_pqm = zm_pqm / (F32(1.0) - zm)[:, None]
            gp = -(gp_pqm.sum(axis=1, dtype=F32) - gp_pqm[:, 13])
            gm = -(gm_pqm.sum(axis=1, dtype=F32) - gm_pqm[:, 13])
        self.mu_m, self.mu_p = mm, mp
        self.zeta_p_pqm, self.zeta_m_pqm = zp_pqm.astype(F32), zm_pqm.astype(F32)
        self.zeta_p, self.zeta_m = zp.astype(F32), zm.astype(F32)
        self.gamma_p_pqm, self.gamma_m_pqm = gp_pqm.astype(F32), gm_pqm.astype(F32)
        self.gamma_p, self.gamma_m = gp.astype(F32), gm.astype(F32)



def projected_points(s, reg: Regression):
    """r_proj = s - phi(s) * n (discretization.py:467, :478, :490, :499)."""
    return (np.asarray(s, F32) - reg.phi[:, None] * reg.normal).astype(F32)


# ----------------------------------------------------------------------------------------
# stencil and boundary (discretization.py:319-364)
# ----------------------------------------------------------------------------------------
def stencil_points(p, h):
    """[ijk, imjk, ipjk, ijmk, ijpk, ijkm, ijkp] (discretization.py:347-353) -> (N, 7, 3)."""
    p = np.asarray(p, F32)
    h = np.asarray(h, F32)
    out = np.repeat(p[:, None, :], 7, axis=1).astype(F32)
    for a in range(3):
        out[:, 1 + 2 * a, a] = p[:, a] - h[a]
        out[:, 2 + 2 * a, a] = p[:, a] + h[a]
    return out


def is_box_boundary(p, h, bounds):
    """``is_box_boundary_point`` (discretization.py:319-333) against the level-set grid bounds."""
    p = np.asarray(p, F32)
    h = np.asarray(h, F32)
    b = np.zeros(p.shape[0], bool)
    for a in range(3):
        tol = F32(1e-6) * h[a]
        b |= np.abs(p[:, a] - F32(bounds[a][0])) < tol
        b |= np.abs(p[:, a] - F32(bounds[a][1])) < tol
    return b


# ----------------------------------------------------------------------------------------
# training data (data_management.py)
# ----------------------------------------------------------------------------------------
def h_level(num_epochs, epoch):
    """``alternate_res_sequentially`` (data_management.py:319-326): zoom = epoch // (E // 4)."""
    return epoch // max(num_epochs // 4, 1)


def h_at_level(h0, level):
    h0 = np.asarray(h0, F32)
    return (h0 * F32(0.5**level)).astype(F32)


def sequential_batches(n_points, batch_size):
    """Slot layout of ``DatasetDict`` for one device (data_management.py:87-159).

    Returns (num_batches, batch_size, n_pad): batches are consecutive ranges of the
    point array; the last partial batch is padded with ``n_pad`` extra points.
    """
    bs = min(batch_size, n_points)
    nb = n_points // bs
    last = n_points % bs
    if last:
        return nb + 1, bs, bs - last
    return nb, bs, 0


# ----------------------------------------------------------------------------------------
# optimizer: clip_by_global_norm(1) -> scale_by_adam -> scale_by_schedule(exp decay) -> scale(-1)
# ----------------------------------------------------------------------------------------
class ChainedAdam:
    """``chained_adam`` (optimizers.py:33-54) with optax 0.1.5 semantics, float32, flat params.

    ``schedule``: "exponential" (``optax.exponential_decay``, non-staircase) or "polynomial"
    (``optax.polynomial_schedule`` with end value 0 and power 1, optimizers.py:25-28: the rate
    falls linearly to 0 over ``transition_steps`` steps and stays there)."""

    def __init__(self, n, lr=1e-3, decay_rate=0.9, transition_steps=1000, max_norm=1.0,
                 b1=0.9, b2=0.999, eps=1e-8, schedule="exponential"):
        self.mu = np.zeros(n, F32)
        self.nu = np.zeros(n, F32)
        self.count = 0
        self.lr, self.rate, self.ts, self.max_norm = F32(lr), F32(decay_rate), transition_steps, F32(max_norm)
        self.b1, self.b2, self.eps = F32(b1), F32(b2), F32(eps)
        self.schedule = schedule

    def step_size(self):
        if self.schedule == "polynomial":
            c = F32(min(max(self.count, 0), self.ts))
            return F32(self.lr * (F32(1) - c / F32(self.ts)))
        return F32(self.lr * self.rate ** F32(self.count / self.ts))

    def update(self, params, grads):
        g = np.asarray(grads, F32)
        gnorm = np.sqrt(np.sum(g.astype(F32) * g, dtype=F32)).astype(F32)
        if not (gnorm < self.max_norm):
            g = (g / gnorm) * self.max_norm
        self.mu = ((F32(1) - self.b1) * g + self.b1 * self.mu).astype(F32)
        self.nu = ((F32(1) - self.b2) * (g * g) + self.b2 * self.nu).astype(F32)
        cnt = self.count + 1
        mu_hat = self.mu / (F32(1) - self.b1 ** F32(cnt))
        nu_hat = self.nu / (F32(1) - self.b2 ** F32(cnt))
        upd = mu_hat / (np.sqrt(nu_hat) + self.eps)
        step = self.step_size()
        upd = (upd * F32(step)) * F32(-1.0)
        self.count = cnt
        return (np.asarray(params, F32) + upd).astype(F32)


class RMSprop:
    """``optax.rmsprop(learning_rate)`` (optimizers.py:82-87; optax 0.1.5: ``scale_by_rms`` with
    decay 0.9, eps 1e-8 and initial scale 0, then ``scale(-learning_rate)``), float32, flat params:
    nu = (1 - decay) g^2 + decay nu; params += -lr g / sqrt(nu + eps)."""

    def __init__(self, n, lr=1e-3, decay=0.9, eps=1e-8):
        self.nu = np.zeros(n, F32)
        self.count = 0
        self.lr, self.decay, self.eps = F32(lr), F32(decay), F32(eps)

    def update(self, params, grads):
        g = np.asarray(grads, F32)
        self.nu = ((F32(1) - self.decay) * (g * g) + self.decay * self.nu).astype(F32)
        upd = (g / np.sqrt(self.nu + self.eps)).astype(F32)
        self.count += 1
        return (np.asarray(params, F32) + (upd * self.lr) * F32(-1.0)).astype(F32)
