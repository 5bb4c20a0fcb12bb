"""CPU oracle, part 2: the parameter-dependent residual, loss and gradient.

TEST INFRASTRUCTURE ONLY (see ``nbm_oracle.py`` for the scope and the parity
status).  The forward restates, literally, ``compute_Ax_and_b_preconditioned_fn``
and ``get_u_mp_by_regression_at_point_fn`` (solvers/poisson/discretization.py:299-519)
and ``Trainer.loss`` (solvers/poisson/trainer.py:892-912) with the preconditioner
disabled (``precond = 1.0``, trainer.py:245-253).  The nonlinear operators N-(u-) V- +
N+(u+) V+ (discretization.py:369) come from the problem's ``nl_m``/``nl_p`` callables
(torch-callable; absent: zero, the reference's default, trainer.py:1007-1017).  The
u^-/u^+ networks restate ``DoubleMLP``
(nn/mlp/MLP.py:93-139): ``hk.Linear`` + tanh per hidden layer, ``Linear(1)`` out,
u = MLP_p(x) where phi(x) >= 0 else MLP_m(x).

The reverse pass is torch.autograd on CPU, standing in for
``jax.value_and_grad(self.loss)`` (trainer.py:786).  It can run in float32
(the reference's precision) or float64 (the FP64 evaluation that every result's
error is stated against).  Geometry and coefficient values always come from
the float32 restatement in ``nbm_oracle.py``, so both precisions take the same
discrete decisions.

Parameter packing (a documented format shared with the CUDA path): one flat
float32 vector, net m first then net p; per net, for each hidden layer
``W[in][out]`` row-major then ``b[out]``; then the output layer ``W[width]``
then ``b[1]``.  This is the haiku pytree order of
``double_mlp/~mlp_{m,p}_fn/linear{,_1,...}`` with ``w`` before ``b``.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

import nbm_oracle as O

F32 = np.float32


@dataclass(frozen=True)
class Arch:
    m_layers: int = 1
    m_width: int = 1
    p_layers: int = 2
    p_width: int = 10
    # learned preconditioner (nn/preconditioner.py:10-35); 0 layers = off
    pre_layers: int = 0
    pre_width: int = 0
    pre_scaling: float = 1.0

    def net(self, which):
        return (self.m_layers, self.m_width) if which == "m" else (self.p_layers, self.p_width)


def net_sizes(layers, width, d_in=3):
    shapes = []
    i = d_in
    for _ in range(layers):
        shapes.append((i, width))
        i = width
    shapes.append((i, 1))
    return shapes


def pre_sizes(arch: Arch):
    return net_sizes(arch.pre_layers, arch.pre_width, 26) if arch.pre_layers > 0 else []


def n_params(arch: Arch):
    tot = 0
    for which in ("m", "p"):
        for a, b in net_sizes(*arch.net(which)):
            tot += a * b + b
    return tot + sum(a * b + b for a, b in pre_sizes(arch))


def unflatten(flat, arch: Arch):
    out = {}
    off = 0
    for which in ("m", "p"):
        layers = []
        for a, b in net_sizes(*arch.net(which)):
            W = flat[off:off + a * b].reshape(a, b)
            off += a * b
            bb = flat[off:off + b]
            off += b
            layers.append((W, bb))
        out[which] = layers
    pre = []
    for a, b in pre_sizes(arch):
        W = flat[off:off + a * b].reshape(a, b)
        off += a * b
        bb = flat[off:off + b]
        off += b
        pre.append((W, bb))
    out["pre"] = pre
    assert off == flat.shape[0]
    return out


def mlp(layers, x):
    h = x
    for W, b in layers[:-1]:
        h = torch.tanh(h @ W + b)
    W, b = layers[-1]
    return (h @ W + b)[..., 0]


def nn_eval(net, x, phi_x):
    """``DoubleMLP.__call__``: MLP_p where phi >= 0 else MLP_m (MLP.py:98)."""
    shp = x.shape[:-1]
    x = x.reshape(-1, 3)
    phi_x = torch.as_tensor(np.asarray(phi_x).reshape(-1))
    sel_p = phi_x >= 0
    out = torch.zeros(x.shape[0], dtype=x.dtype)
    if bool(sel_p.any()):
        out = out.index_put((sel_p.nonzero()[:, 0],), mlp(net["p"], x[sel_p]))
    sel_m = ~sel_p
    if bool(sel_m.any()):
        out = out.index_put((sel_m.nonzero()[:, 0],), mlp(net["m"], x[sel_m]))
    return out.reshape(shp)


class Problem:
    """Grid level set plus coefficient callables, all evaluated in float32 numpy.

    ``phi`` is the trilinear interpolant of the (perturbed) level-set samples; the
    coefficient callables take coordinates as an array of shape (3, M).
    """

    def __init__(self, phi_values, lvl_x, lvl_y, lvl_z, fns):
        self.phi = O.Trilinear(phi_values, lvl_x, lvl_y, lvl_z)
        self.bounds = [(F32(np.min(a)), F32(np.max(a))) for a in (lvl_x, lvl_y, lvl_z)]
        self.fns = fns

    def co(self, name, pts):
        pts = np.asarray(pts, F32)
        shp = pts.shape[:-1]
        flat = pts.reshape(-1, 3)
        v = np.asarray(self.fns[name](flat.T), F32)
        return np.broadcast_to(v, flat.shape[:1]).astype(F32).reshape(shp)


class ResidualGeometry:
    """All parameter-independent quantities of the residual at points ``p`` and spacing ``h``."""

    def __init__(self, prob: Problem, p, h):
        p = np.asarray(p, F32)
        h = np.asarray(h, F32)
        N = p.shape[0]
        self.p, self.h, self.N = p, h, N
        phi = prob.phi
        self.bnd = O.is_box_boundary(p, h, prob.bounds)
        geo = O.CellGeometry(phi, p, h)
        faces = O.face_centres(p, h)
        self.mu_m_faces = prob.co("mu_m", faces)
        self.mu_p_faces = prob.co("mu_p", faces)
        self.coeffs = O.face_coefficients(geo, self.mu_m_faces, self.mu_p_faces)
        self.crossed_p = geo.crossed
        self.beta_int = O.interface_integral(geo, lambda q: prob.co("beta", q))
        self.k_m, self.k_p = prob.co("k_m", p), prob.co("k_p", p)
        self.f_m, self.f_p = prob.co("f_m", p), prob.co("f_p", p)
        self.g = prob.co("g", p)
        self.nl_m, self.nl_p = prob.fns.get("nl_m"), prob.fns.get("nl_p")
        self.stencil = O.stencil_points(p, h)  # (N,7,3)
        st = self.stencil.reshape(-1, 3)
        self.crossed_s = O.is_crossed(phi, st, h).reshape(N, 7)
        self.phi_s = phi(st).reshape(N, 7)
        # crossed stencil points -> regression data
        idx = np.nonzero(self.crossed_s.reshape(-1) == 0)[0]
        self.x_idx = idx
        s = st[idx]
        self.x_mu_m, self.x_mu_p = prob.co("mu_m", s), prob.co("mu_p", s)
        reg = O.Regression(phi, s, h, self.x_mu_m, self.x_mu_p)
        self.reg = reg
        rp = O.projected_points(s, reg)
        self.x_rproj = rp
        self.x_alpha = prob.co("alpha", rp)
        self.x_beta = prob.co("beta", rp)
        self.x_mu_m_r = prob.co("mu_m", rp)
        self.x_mu_p_r = prob.co("mu_p", rp)

    @property
    def n_crossed_stencil(self):
        return int(self.x_idx.shape[0])


def _t(a, dtype):
    return torch.as_tensor(np.asarray(a)).to(dtype)


def residual(flat_params, arch: Arch, rg: ResidualGeometry, dtype=torch.float32):
    """Per-point residual lhs/diag - rhs/diag (nan_to_num'd), shape (N,)."""
    net = unflatten(flat_params, arch)
    N = rg.N
    T = lambda a: _t(a, dtype)  # noqa: E731
    st = T(rg.stencil)
    u_s = nn_eval(net, st, rg.phi_s)  # (N,7)
    cr = T(rg.crossed_s)
    zero = torch.zeros((), dtype=dtype)
    u_m = torch.where(cr == -1, u_s, zero)
    u_p = torch.where(cr == 1, u_s, zero)
    if rg.n_crossed_stencil:
        reg = rg.reg
        idx = torch.as_tensor(rg.x_idx)
        u = u_s.reshape(-1)[idx]
        cube = nn_eval(net, T(reg.vertices), reg.phi_vertices)  # (E,27)
        delta = T(reg.phi)
        a, b = T(rg.x_alpha), T(rg.x_beta)
        bm = b / T(rg.x_mu_m_r)
        bp = b / T(rg.x_mu_p_r)

        def extrap(G_pqm, g):
            G_pqm, g = T(G_pqm), T(g)
            return -(G_pqm * cube).sum(1) + (1.0 - g + G_pqm[:, 13]) * u

        # mu^- > mu^+ branch (discretization.py:465-486)
        um_A = extrap(reg.gamma_m_pqm, reg.gamma_m) + (-1.0 * (1.0 - T(reg.gamma_m))) * (a + delta * bp)
        up_A = extrap(reg.zeta_m_pqm, reg.zeta_m) + (a + delta * bp)
        um_1 = torch.where(delta > 0, um_A, u)
        up_1 = torch.where(delta > 0, u, up_A)
        # mu^+ >= mu^- branch (discretization.py:488-509)
        um_B = extrap(reg.zeta_p_pqm, reg.zeta_p) + (-1.0) * (a + delta * bm)
        up_B = extrap(reg.gamma_p_pqm, reg.gamma_p) + (1.0 - T(reg.gamma_p)) * (a + delta * bm)
        um_2 = torch.where(delta > 0, um_B, u)
        up_2 = torch.where(delta > 0, u, up_B)
        mbig = T(reg.mu_m) > T(reg.mu_p)
        um_x = torch.where(mbig, um_1, um_2)
        up_x = torch.where(mbig, up_1, up_2)
        u_m = u_m.reshape(-1).index_put((idx,), um_x).reshape(N, 7)
        u_p = u_p.reshape(-1).index_put((idx,), up_x).reshape(N, 7)

    c = T(rg.coeffs)
    Vm, Vp = c[:, 12], c[:, 13]
    km, kp = T(rg.k_m), T(rg.k_p)
    se = ((((c[:, 0] + c[:, 2]) + c[:, 4]) + c[:, 6]) + c[:, 8]) + c[:, 10]
    so = ((((c[:, 1] + c[:, 3]) + c[:, 5]) + c[:, 7]) + c[:, 9]) + c[:, 11]
    lhs = km * Vm * u_m[:, 0]
    lhs = lhs + kp * Vp * u_p[:, 0]
    if rg.nl_m is not None or rg.nl_p is not None:  # discretization.py:369
        nm = rg.nl_m(u_m[:, 0]) if rg.nl_m is not None else torch.zeros_like(Vm)
        npl = rg.nl_p(u_p[:, 0]) if rg.nl_p is not None else torch.zeros_like(Vp)
        lhs = lhs + nm * Vm + npl * Vp
    lhs = lhs + se * u_m[:, 0] + so * u_p[:, 0]
    for j in range(1, 7):
        lhs = lhs + (-1.0 * c[:, 2 * (j - 1)] * u_m[:, j] - c[:, 2 * (j - 1) + 1] * u_p[:, j])
    diag = kp * Vp + km * Vm + se + so
    rhs = T(rg.f_m) * Vm + T(rg.f_p) * Vp + T(rg.beta_int)
    h = rg.h
    V = T(F32(h[0] * h[1] * h[2]))
    bnd = torch.as_tensor(rg.bnd)
    lhs = torch.where(bnd, u_s[:, 0] * V, lhs)
    diag = torch.where(bnd, V.expand(N), diag)
    rhs = torch.where(bnd, T(rg.g) * V, rhs)
    r = torch.nan_to_num(lhs / diag) - torch.nan_to_num(rhs / diag)
    if arch.pre_layers > 0:
        # precond = 0.5 + s * sigmoid(Dense(tanh(...)(coeffs_))) multiplies lhs/diag and rhs/diag
        # (discretization.py:339, :419-420; nn/preconditioner.py:21-35)
        P = 0.5 + arch.pre_scaling * torch.sigmoid(mlp(net["pre"], T(rg.coeffs)))
        r = P * r
    return r


def loss(flat_params, arch: Arch, rg: ResidualGeometry, dtype=torch.float32):
    """``Trainer.loss`` = mean(optax.l2_loss(lhs, rhs)) = mean(0.5*(lhs-rhs)^2) (trainer.py:892-912)."""
    r = residual(flat_params, arch, rg, dtype)
    return torch.mean(0.5 * r * r)


def loss_and_grad(flat_np, arch: Arch, rg: ResidualGeometry, dtype=torch.float32):
    flat = torch.tensor(np.asarray(flat_np), dtype=dtype, requires_grad=True)
    L = loss(flat, arch, rg, dtype)
    (g,) = torch.autograd.grad(L, flat)
    return float(L.detach()), g.detach().numpy()


def init_params(arch: Arch, seed=0):
    """Haiku-style init: hidden W ~ TruncatedNormal(0.1), output W ~ TruncatedNormal(1/sqrt(fan_in)), b = 0.

    (MLP.py:65, :70, :112-115; hk.Linear default w_init for the output layer.)  The
    draw uses numpy's generator, not jax's PRNG.
    """
    rng = np.random.default_rng(seed)
    parts = []
    for which in ("m", "p"):
        shapes = net_sizes(*arch.net(which))
        for li, (a, b) in enumerate(shapes):
            std = 0.1 if li < len(shapes) - 1 else 1.0 / np.sqrt(a)
            w = rng.standard_normal((a, b))
            while np.any(np.abs(w) > 2.0):
                bad = np.abs(w) > 2.0
                w[bad] = rng.standard_normal(int(bad.sum()))
            parts.append((w * std / 0.87962566103423978).astype(F32).ravel())
            parts.append(np.zeros(b, F32))
    for a, b in pre_sizes(arch):  # flax Dense: glorot_uniform kernels, zero biases (preconditioner.py:18-35)
        lim = np.sqrt(6.0 / (a + b))
        parts.append(rng.uniform(-lim, lim, (a, b)).astype(F32).ravel())
        parts.append(np.zeros(b, F32))
    return np.concatenate(parts).astype(F32)


def evaluate_solution(flat_np, arch: Arch, prob: Problem, pts, dtype=torch.float32):
    """``Trainer.evaluate_solution_fn`` (trainer.py:836-844)."""
    net = unflatten(torch.as_tensor(np.asarray(flat_np)).to(dtype), arch)
    pts = np.asarray(pts, F32)
    with torch.no_grad():
        return nn_eval(net, _t(pts, dtype), prob.phi(pts)).numpy()
