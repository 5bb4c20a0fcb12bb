"""Writes golden vectors computed by the reference's own residual code.

Run from the repository root, where the reference checkout is readable::

    python tests/golden/make_reference_golden.py [reference checkout [case ...]]

Each case imports the reference's unmodified ``solvers/poisson/discretization.py``,
``geometry/geometric_integrations_per_point.py``, ``geometry/level_set.py`` and
``domain/interpolate.py`` on the numpy stand-in for jax (``oracle/refjax.py``) through
``oracle/ref_harness.py``, and records, for a seeded subset of the grid points of one stencil
level:

* ``phi``       the perturbed level-set samples on the grid (the interpolant's input; the GPU
                tests feed exactly these samples to the CUDA path)
* ``ids``       the batch (indices into the grid's C-order points)
* ``params``    the flat parameter vector (float32)
* ``lhs_rhs``   per point [lhs/diag, rhs/diag] of ``compute_Ax_and_b_preconditioned_fn``
                (discretization.py:299-423), float32 (jax_enable_x64 off)
* ``coeff26``   the 26 cell values of ``compute_cell_faces_areas_values`` (geom_pp.py:464-1009)
* ``beta_int``  ``integrate_over_interface_at_point`` (geom_pp.py:383-461)
* ``crossed``   ``is_point_cell_crossed_by_interface`` (geom_pp.py:203-263)
* ``loss32``    ``Trainer.loss`` (trainer.py:892-912) with x64 off
* ``loss64``    the same with jax_enable_x64 on and float64 parameters
* ``dirs``, ``dloss64``  three random unit directions in parameter space and the directional
                derivative of the x64 loss along each, by fourth-order central differences
                (step 1e-3); they pin the gradient.

The problems are the product's restatements in ``dips_gb300/problems.py`` (coefficient
callables wrapped as per-point functions, as ``trainer.setup`` vmaps them); two of them are the
reference's own manufactured problems (``tests/confs/experiment_configs.py``), and
``tests/test_reference_problems.py`` checks those restatements against the reference's callables.
"""

from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for sub in ("oracle", "jax-dips_gb300"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

F32 = np.float32

# where the reference checkout is read in the container that writes these fixtures
DEFAULT_REFERENCE = "/root/reference"

# name: (problem, grid n, network (m_layers, m_width, p_layers, p_width), level, points near / far)
CASES = {
    "sphere16_1x1_2x10_l0": ("sphere", 16, (1, 1, 2, 10), 0, 160, 96),
    "sphere16_3x32_l1": ("sphere", 16, (3, 32, 3, 32), 1, 160, 96),
    "star16_2x16_l0": ("star", 16, (2, 16, 2, 16), 0, 160, 96),
    "refsphere16_3x32_l0": ("refsphere", 16, (3, 32, 3, 32), 0, 160, 96),
    "refstar16_2x16_l0": ("refstar", 16, (2, 16, 2, 16), 0, 160, 96),
    "sphere_mu10_1_16_3x32_l0": ("sphere_mu10_1", 16, (3, 32, 3, 32), 0, 160, 96),
    "blob16_4x64_l0": ("blob", 16, (4, 64, 4, 64), 0, 160, 96),
    "lpbe16_2x16_l0": ("lpbe", 16, (2, 16, 2, 16), 0, 160, 96),
    "sphere16_sinh_3x32_l0": ("sphere_sinh", 16, (3, 32, 3, 32), 0, 160, 96),
}


def lpbe_spheres(seed=0, n=60):
    """A small seeded LPBE molecule: n spheres (centres U[-0.6,0.6]^3, radii U[0.05,0.12],
    charges in {-1,0,1})."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.6, 0.6, (n, 3)).astype(F32)
    r = rng.uniform(0.05, 0.12, n).astype(F32)
    q = rng.integers(-1, 2, n).astype(F32)
    return c, r, q


def problem(name):
    from dips_gb300 import problems

    if name == "sphere":
        return problems.sphere_problem()
    if name == "sphere_mu10_1":
        return problems.sphere_problem(mu_m=10.0, mu_p=1.0)
    if name == "star":
        return problems.star_problem()
    if name == "refsphere":
        return problems.reference_sphere_problem()
    if name == "refstar":
        return problems.reference_star_problem()
    if name == "blob":
        return problems.blob_problem()
    if name == "lpbe":
        return problems.lpbe_problem(*lpbe_spheres())
    if name == "sphere_sinh":  # the sphere with nonlinear operators N-(u) = 300 sinh(u), N+(u) = 100 sinh(u)
        from dips_gb300 import nonlinear

        return dict(problems.sphere_problem(), nl_m=nonlinear.Sinh(300.0), nl_p=nonlinear.Sinh(100.0))
    raise KeyError(name)


def select_ids(phi, dx, near, far, seed=0):
    rng = np.random.default_rng(seed)
    close = np.nonzero(np.abs(phi) < 2.5 * dx)[0]
    rest = np.nonzero(np.abs(phi) >= 2.5 * dx)[0]
    a = rng.choice(close, min(near, close.size), replace=False)
    b = rng.choice(rest, min(far, rest.size), replace=False)
    return np.sort(np.concatenate([a, b])).astype(np.int32)


def case_params(arch, seed=0):
    import nbm_loss as L

    p = L.init_params(L.Arch(*arch), seed)
    rng = np.random.default_rng(seed + 1000)
    return (p + F32(0.02) * rng.standard_normal(p.shape).astype(F32)).astype(F32)


def run_case(args):
    ref_root, name = args
    import ref_harness as H

    import nbm_loss as L
    import nbm_oracle as O

    prob_name, n, arch, level, near, far = CASES[name]
    t0 = time.time()
    mods = H.load(ref_root, x64=False)
    import jax
    import jax.numpy as jnp
    import refjax

    prob = problem(prob_name)
    x = jnp.linspace(-1.0, 1.0, n, dtype=jnp.float32)
    gs = mods["mesh"].construct(3)[0](x, x, x)
    R = np.asarray(gs.R, F32)
    phi = O.perturb(np.asarray(prob["phi"](R.T), F32))
    dx = F32(np.asarray(gs.dx))
    h = F32(dx * F32(0.5 ** level))
    ids = select_ids(phi, dx, near, far)
    pts = R[ids]
    a = L.Arch(*arch)
    flat = case_params(arch)
    if prob_name == "sphere_sinh":
        # output biases +0.8 (u-) and -0.6 (u+): u of order one, where sinh is far from linear
        sizes_m = L.net_sizes(*a.net("m"))
        n_m = sum(i * o + o for i, o in sizes_m)
        n_p = sum(i * o + o for i, o in L.net_sizes(*a.net("p")))
        flat = flat.copy()
        flat[n_m - 1] += F32(0.8)
        flat[n_m + n_p - 1] -= F32(0.6)
    out = dict(name=np.array(name), problem=np.array(prob_name), n=np.int32(n), level=np.int32(level),
               arch=np.array(arch, np.int32), phi=phi, ids=ids, params=flat, h=h)

    def build(dtype):
        phi_fn = mods["interpolate"].multilinear_interpolation(jnp.asarray(phi), gs)
        fns = {k: H.per_point(prob[k], dtype) for k in ("mu_m", "mu_p", "k_m", "k_p", "f_m", "f_p", "alpha",
                                                         "beta", "g")}
        fns["u0"] = lambda r: 0.0
        for k in ("nl_m", "nl_p"):
            if k in prob:
                fns[k] = prob[k]
        ssf = H.sim_state_fn_from(mods, fns, phi_fn)
        return H.make_harness(mods)(gs, ssf, a)

    # ---- x64 off: the reference's precision
    hz = build(F32)
    P = jnp.asarray(pts)
    loss32, lr = hz.loss({"flat": flat}, P, h, h, h)
    out["loss32"] = np.float32(loss32)
    out["lhs_rhs"] = lr.astype(F32)
    c26, bint, cr = [], [], []
    for i in range(pts.shape[0]):
        p = jnp.asarray(pts[i])
        c26.append(np.asarray(refjax._raw(hz.compute_face_centroids_values_plus_minus_at_point(p, h, h, h)), F32))
        bint.append(np.asarray(refjax._raw(hz.beta_integrate_over_interface_at_point(p, h, h, h)), F32))
        cr.append(np.asarray(refjax._raw(hz.is_cell_crossed_by_interface(p, h, h, h))))
    out["coeff26"] = np.stack(c26).reshape(-1, 26).astype(F32)
    out["beta_int"] = np.stack(bint).reshape(-1).astype(F32)
    out["crossed"] = np.stack(cr).reshape(-1).astype(np.float32)
    t1 = time.time()

    # ---- x64 on: float64 parameters, loss and directional derivatives
    refjax.set_x64(True)
    hz64 = build(np.float64)
    P64 = jnp.asarray(pts)
    f64 = flat.astype(np.float64)

    def L64(v):
        return float(hz64.loss({"flat": v}, P64, h, h, h)[0])

    out["loss64"] = np.float64(L64(f64))
    rng = np.random.default_rng(7)
    dirs, ders = [], []
    eps = 1e-3
    for _ in range(3):
        v = rng.standard_normal(f64.shape)
        v /= np.linalg.norm(v)
        vals = [L64(f64 + s * eps * v) for s in (-2, -1, 1, 2)]
        dirs.append(v.astype(F32))
        ders.append((vals[0] - 8 * vals[1] + 8 * vals[2] - vals[3]) / (12 * eps))
    refjax.set_x64(False)
    out["dirs"] = np.stack(dirs)
    out["dloss64"] = np.array(ders, np.float64)
    path = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(path, **out)
    del jax
    return name, pts.shape[0], float(loss32), out["loss64"], time.time() - t0, t1 - t0


# the discrete FV operator of a nodal vector (the plain method's system): name -> (problem, n)
FV_CASES = {
    "fvop_sphere16": ("sphere", 16),
    "fvop_refsphere16": ("refsphere", 16),
}


def fv_rows(n, phi, dx, seed=0):
    """Rows of the discrete-operator fixture: 96 in the two lowest node layers of some axis
    (where the reference's interpolant extrapolates the first cell), 96 within 2.5 dx of the
    interface, 64 others."""
    rng = np.random.default_rng(seed)
    ijk = np.stack(np.unravel_index(np.arange(n ** 3), (n, n, n)), 1)
    low = np.nonzero((ijk <= 1).any(1))[0]
    near = np.nonzero((np.abs(phi) < 2.5 * dx) & ~(ijk <= 1).any(1))[0]
    a = rng.choice(low, 96, replace=False)
    b = rng.choice(near, min(96, near.size), replace=False)
    rest = np.setdiff1d(np.arange(n ** 3), np.concatenate([a, b]))
    c = rng.choice(rest, 64, replace=False)
    return np.sort(np.concatenate([a, b, c])).astype(np.int32)


def run_fv_case(args):
    """``Trainer.residual_vector`` (trainer.py:883-890) of two nodal vectors -- seeded normal
    values and the exact solution at the nodes -- at a seeded set of rows, float32."""
    ref_root, name = args
    import ref_harness as H

    import nbm_loss as L
    import nbm_oracle as O

    prob_name, n = FV_CASES[name]
    t0 = time.time()
    mods = H.load(ref_root, x64=False)
    import jax.numpy as jnp

    from dips_gb300 import problems

    prob = problem(prob_name)
    x = jnp.linspace(-1.0, 1.0, n, dtype=jnp.float32)
    gs = mods["mesh"].construct(3)[0](x, x, x)
    R = np.asarray(gs.R, F32)
    phi = O.perturb(np.asarray(prob["phi"](R.T), F32))
    dx = F32(np.asarray(gs.dx))
    rows = fv_rows(n, phi, dx)
    phi_fn = mods["interpolate"].multilinear_interpolation(jnp.asarray(phi), gs)
    fns = {k: H.per_point(prob[k], F32) for k in ("mu_m", "mu_p", "k_m", "k_p", "f_m", "f_p", "alpha", "beta", "g")}
    fns["u0"] = lambda r: 0.0
    hz = H.make_harness(mods)(gs, H.sim_state_fn_from(mods, fns, phi_fn), L.Arch(1, 1, 2, 10))
    u_rand = np.random.default_rng(5).standard_normal(n ** 3).astype(F32)
    u_exact = problems.exact_solution(prob, R).astype(F32)
    out = dict(name=np.array(name), problem=np.array(prob_name), n=np.int32(n), phi=phi, rows=rows,
               u_rand=u_rand, u_exact=u_exact)
    P = jnp.asarray(R[rows])
    for key, u in (("res_rand", u_rand), ("res_exact", u_exact)):
        out[key] = hz.residual_vector_rows(gs, jnp.asarray(u), P, dx, dx, dx).astype(F32)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
    return name, rows.size, float(np.abs(out["res_rand"]).max()), float(np.abs(out["res_exact"]).max()), \
        time.time() - t0


# the per-device batch layout of DatasetDict(x, batch_size, num_gpus) (data_management.py:79-159):
# (points, batch size, devices)
DATA_CASES = ((1000, 128, 1), (1000, 128, 2), (1000, 100, 3), (1024, 256, 4), (999, 1000, 2),
              (4096, 4096, 1), (37, 8, 3), (125, 7, 1), (50, 7, 4))
PAD = -123.0  # stands for the padding points in ref_dataset_layout.npz


def run_data_case(ref_root):
    """``ref_dataset_layout.npz``: ``DatasetDict(x, batch_size, num_gpus).batched_data`` of the
    reference for each of DATA_CASES, x[i] = (3i, 3i+1, 3i+2)/7 so that every point is
    identifiable.  The padding points are drawn by ``generate_random_points_like`` with
    ``jax.random.PRNGKey(0)``, which the stand-in cannot reproduce; that one function is replaced by
    one returning rows of PAD, so the fixture records where the padding goes (its values are a
    documented deviation: the product draws them with numpy)."""
    import ref_harness as H
    import refjax

    dm = H.load_data_management(ref_root)
    dm.generate_random_points_like = lambda x, k: refjax._wrap(np.full((k, 3), PAD, F32))
    out = {"cases": np.array(DATA_CASES, np.int64), "pad": np.float32(PAD)}
    for i, (n, bs, g) in enumerate(DATA_CASES):
        x = np.arange(3 * n, dtype=F32).reshape(n, 3) / F32(7.0)
        d = dm.DatasetDict(refjax._wrap(x), bs, num_gpus=g)
        b = np.asarray(refjax._raw(d.batched_data), F32)
        out[f"batched_{i}"] = b if g > 1 else b[None]
    return out


def run_interp_case(ref_root, n=16):
    """``ref_interp_nodal16.npz``: the reference's ``multilinear_interpolation`` (interpolate.py:
    906-1021) and ``nonoscillatory_quadratic_interpolation`` (:572-759) of a seeded nodal field on
    the n^3 grid over [-1, 1]^3, at 650 seeded points: inside the box, in the first and last cells
    of each axis (where both clamp their cell index and extrapolate), beyond the box, and on nodes."""
    import ref_harness as H
    import refjax

    mods = H.load(ref_root, x64=False)
    import jax.numpy as jnp

    x = jnp.linspace(-1.0, 1.0, n, dtype=jnp.float32)
    gs = mods["mesh"].construct(3)[0](x, x, x)
    R = np.asarray(refjax._raw(gs.R), F32)
    rng = np.random.default_rng(3)
    u = (np.sin(3 * R[:, 0]) * np.cos(2 * R[:, 1]) + R[:, 2] ** 2 + 0.1 * rng.standard_normal(n ** 3)).astype(F32)
    pts = np.concatenate([rng.uniform(-1, 1, (300, 3)), rng.uniform(-1.0, -0.8, (100, 3)),
                          rng.uniform(0.8, 1.0, (100, 3)), rng.uniform(-1.2, 1.2, (100, 3)),
                          R[rng.choice(n ** 3, 50)]]).astype(F32)
    tri = mods["interpolate"].multilinear_interpolation(jnp.asarray(u), gs)
    quad = mods["interpolate"].nonoscillatory_quadratic_interpolation(jnp.asarray(u), gs)
    return {"n": np.int32(n), "u": u, "pts": pts,
            "trilinear": np.asarray(refjax._raw(tri(jnp.asarray(pts))), F32).reshape(-1),
            "quadratic": np.asarray(refjax._raw(quad(jnp.asarray(pts))), F32).reshape(-1)}


def main(argv):
    ref_root = argv[1] if len(argv) > 1 else DEFAULT_REFERENCE
    names = argv[2:] or (list(CASES) + list(FV_CASES) + ["dataset_layout", "interp_nodal16"])
    if "interp_nodal16" in names:
        np.savez_compressed(os.path.join(HERE, "ref_interp_nodal16.npz"), **run_interp_case(ref_root))
        print("interp_nodal16", flush=True)
    if "dataset_layout" in names:
        np.savez_compressed(os.path.join(HERE, "ref_dataset_layout.npz"), **run_data_case(ref_root))
        print("dataset_layout: %d cases" % len(DATA_CASES), flush=True)
    fv = [nm for nm in names if nm in FV_CASES]
    names = [nm for nm in names if nm in CASES]
    ctx = mp.get_context("spawn")
    if fv:
        with ctx.Pool(len(fv)) as pool:
            for r in pool.imap_unordered(run_fv_case, [(ref_root, nm) for nm in fv]):
                print("%-28s rows %4d  max|r(u_rand)| %.4e  max|r(u_exact)| %.4e  %.0f s" % r, flush=True)
    if not names:
        return
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(len(names), max(1, (os.cpu_count() or 2) - 1))) as pool:
        for r in pool.imap_unordered(run_case, [(ref_root, nm) for nm in names]):
            print("%-28s points %4d  loss32 %.7e  loss64 %.9e  %.0f s (x32 part %.0f s)" % r, flush=True)


if __name__ == "__main__":
    main(sys.argv)
