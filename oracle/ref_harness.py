"""Runs the reference's own residual code (unmodified source files) on the numpy stand-in for jax.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module.  It is used by
``tests/golden/make_reference_golden.py`` to write golden vectors produced by the reference's
code, and by a CPU test that regenerates a few of them when the reference's sources are present.

The reference's files are imported from the reference checkout as they are; the only code here
restates the few ``Trainer`` methods that the residual path calls on ``self`` (the rest of
``solvers/poisson/trainer.py`` needs optax, haiku and flax, which are not installed):

* ``solution_at_point_fn``  -- trainer.py:850-855 (``forward.apply(params, None, r, phi)``)
* ``evaluate_solution_fn``  -- trainer.py:836-844 (vmap of the network over points)
* ``precond_fn``            -- trainer.py:245-253 with the preconditioner disabled (returns 1.0)
* ``loss``                  -- trainer.py:892-912: mean of ``optax.l2_loss(lhs, rhs)``,
  i.e. mean of 0.5 (lhs - rhs)^2 (optax 0.1.5)
* the u-/u+ networks        -- ``DoubleMLP`` (nn/mlp/MLP.py:93-139): ``hk.Linear`` + tanh per
  hidden layer, ``Linear(1)`` out, u = MLP_p(x) where phi(x) >= 0 else MLP_m(x), with the
  parameters in the flat layout of ``nbm_loss.py`` (haiku tree order, ``w`` before ``b``).

Pure, parameter-independent per-point functions of the reference (cell geometry, interface
integral, regression coefficients, crossing test, the phi interpolant) are memoised by their
exact argument bytes, so that repeated evaluations -- the same stencil point seen from
neighbouring training points, or the loss re-evaluated at perturbed parameters for finite
differences -- run the reference's code once.  Memoising a pure function does not change any
value.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import refjax  # noqa: E402


def load(ref_root, x64=False):
    """Install the stand-in and import the reference modules from ``ref_root``."""
    refjax.install(x64=x64)
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    import importlib

    mods = {}
    for name in ("jax_dips.domain.interpolate", "jax_dips.domain.mesh", "jax_dips.geometry.level_set",
                 "jax_dips.geometry.geometric_integrations_per_point", "jax_dips.solvers.simulation_states",
                 "jax_dips.solvers.poisson.discretization", "tests.confs.experiment_configs"):
        mods[name.split(".")[-1]] = importlib.import_module(name)
    return mods


def load_data_management(ref_root):
    """Install the stand-in and import the reference's ``data/data_management.py`` (``DatasetDict``,
    the batching of the training points).  That module also imports ``utils/conversions.py``
    (dlpack converters between jax and torch, and NVIDIA warp helpers), which the batching code
    does not use and which cannot be imported without jaxlib and warp: a module whose functions
    raise stands in for it."""
    import importlib
    import types

    refjax.install(x64=False)
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    name = "jax_dips.utils.conversions"
    if name not in sys.modules:
        stub = types.ModuleType(name)

        def _unavailable(*a, **k):
            raise NotImplementedError(name + " is not available on the stand-in")

        stub.jax_to_torch = stub.torch_to_jax = _unavailable
        sys.modules[name] = stub
    return importlib.import_module("jax_dips.data.data_management")


def _key(*args):
    parts = []
    for a in args:
        x = np.asarray(refjax._raw(a))
        parts.append((x.dtype.str, x.shape, x.tobytes()))
    return tuple(parts)


def memoise(fn):
    cache = {}

    def f(*args):
        k = _key(*args)
        v = cache.get(k)
        if v is None:
            v = fn(*args)
            cache[k] = v
        return v

    f.cache = cache
    return f


def memoise_rows(fn):
    """Memoise a function of a point array (M, 3) row by row (the reference's vmapped interpolant)."""
    cache = {}

    def f(R):
        R = np.asarray(refjax._raw(R))
        if R.ndim == 1:
            return f(R[None])[0]
        out = [None] * R.shape[0]
        missing = []
        for i in range(R.shape[0]):
            v = cache.get(R[i].tobytes())
            if v is None:
                missing.append(i)
            else:
                out[i] = v
        if missing:
            vals = np.asarray(refjax._raw(fn(refjax._wrap(R[missing]))))
            for j, i in enumerate(missing):
                cache[R[i].tobytes()] = vals[j]
                out[i] = vals[j]
        return refjax._wrap(np.stack(out))

    f.cache = cache
    return f


class DoubleMLP:
    """``DoubleMLP`` (nn/mlp/MLP.py:93-139) over the flat parameter vector of ``nbm_loss.py``."""

    def __init__(self, arch):
        self.arch = arch

    def layers(self, flat, which, dtype):
        import nbm_loss as L

        off = 0
        out = {}
        for w in ("m", "p"):
            ls = []
            for a, b in L.net_sizes(*self.arch.net(w)):
                W = np.asarray(flat[off:off + a * b], dtype).reshape(a, b)
                off += a * b
                bb = np.asarray(flat[off:off + b], dtype)
                off += b
                ls.append((W, bb))
            out[w] = ls
        return out[which]

    def apply(self, params, rng, x, phi_x):
        """u(x) for one point (x[3], phi scalar) or a batch (x[N,3], phi[N])."""
        flat = params["flat"]
        xr = np.asarray(refjax._raw(x))
        dt = np.result_type(xr.dtype, np.asarray(flat).dtype)  # hk.Linear promotes x to the params' type
        xr = xr.astype(dt)
        pr = np.asarray(refjax._raw(phi_x))

        def mlp(which):
            h = xr
            ls = self.layers(flat, which, dt)
            for W, b in ls[:-1]:
                h = np.tanh(h @ W + b).astype(dt)
            W, b = ls[-1]
            return (h @ W + b).astype(dt)

        up, um = mlp("p"), mlp("m")
        if xr.ndim == 2:
            pr = pr.reshape(-1, 1)
        return refjax._wrap(np.where(pr >= 0, up, um))

    apply.__refjax_batched__ = True


DoubleMLP.apply.__refjax_batched__ = True


def make_harness(mods):
    Discretization = mods["discretization"].Discretization

    class Harness(Discretization):
        """The reference's ``Discretization`` with the ``Trainer`` methods its residual calls."""

        def __init__(self, lvl_gstate, sim_state_fn, arch):
            super().__init__(lvl_gstate, None, sim_state_fn, precondition=1, algorithm=0)
            self.forward = DoubleMLP(arch)
            # pure per-point functions: memoised by argument bytes (values unchanged)
            self.phi_interp_fn = memoise_rows(self.phi_interp_fn)
            self.is_cell_crossed_by_interface = memoise(self.is_cell_crossed_by_interface)
            self.compute_face_centroids_values_plus_minus_at_point = memoise(
                self.compute_face_centroids_values_plus_minus_at_point)
            self.beta_integrate_over_interface_at_point = memoise(self.beta_integrate_over_interface_at_point)
            self.get_regression_coeffs_at_point = memoise(self.get_regression_coeffs_at_point)

        # post-processing methods that Discretization.__init__ binds (discretization.py:149-156);
        # they are Trainer methods (trainer.py:914-957) and not on the residual path
        def compute_normal_gradient_solution_mp_on_interface_neural_network(self, *a):
            raise NotImplementedError

        def compute_gradient_solution_mp_neural_network(self, *a):
            raise NotImplementedError

        def compute_normal_gradient_solution_on_interface_neural_network(self, *a):
            raise NotImplementedError

        def compute_gradient_solution_neural_network(self, *a):
            raise NotImplementedError

        # trainer.py:850-855
        def solution_at_point_fn(self, params, r_point, phi_point):
            return self.forward.apply(params, None, r_point, phi_point).reshape(())

        # trainer.py:836-844
        def evaluate_solution_fn(self, params, R_flat):
            phi_flat = self.phi_interp_fn(R_flat)
            return self.forward.apply(params, None, R_flat, phi_flat)

        # trainer.py:245-253, preconditioner disabled
        def precond_fn(self, params, coeffs):
            return 1.0

        def lhs_rhs(self, params, points, dx, dy, dz):
            jax = sys.modules["jax"]
            return jax.vmap(self.compute_Ax_and_b_fn, (None, 0, None, None, None))(params, points, dx, dy, dz)

        # trainer.py:883-890 at chosen rows: lhs/diag - rhs/diag of compute_Ax_and_b_discrete_fn
        # (discretization.py:522-741) for the nodal vector u on eval_gstate
        def residual_vector_rows(self, eval_gstate, u, points, dx, dy, dz):
            jax = sys.modules["jax"]
            lr = jax.vmap(self.compute_Ax_and_b_discrete_fn, (None, None, 0, None, None, None))(
                eval_gstate, u, points, dx, dy, dz)
            lr = np.asarray(refjax._raw(lr))
            lr = lr.reshape(lr.shape[0], 2)
            return lr[:, 0] - lr[:, 1]

        # trainer.py:892-912
        def loss(self, params, points, dx, dy, dz):
            lr = np.asarray(refjax._raw(self.lhs_rhs(params, points, dx, dy, dz)))
            lr = lr.reshape(lr.shape[0], 2)  # per point [lhs/diag, rhs/diag], each of shape (1,)
            lhs, rhs = lr[:, 0], lr[:, 1]
            half = lr.dtype.type(0.5)
            return np.mean(half * (lhs - rhs) ** 2, dtype=lr.dtype), lr

    return Harness


def sim_state_fn_from(mods, fns, phi_fn):
    """``PoissonSimStateFn`` as ``trainer.setup`` builds it (trainer.py:995-1031): every
    per-point callable vmapped; the nonlinear operators ``fns["nl_m"]``/``fns["nl_p"]`` passed
    as they are (called on the scalar u at a point, discretization.py:369), zero when absent."""
    jax = sys.modules["jax"]
    SS = mods["simulation_states"].PoissonSimStateFn
    v = jax.vmap

    def zero(x):
        return 0.0

    nl_m = fns.get("nl_m") or zero
    nl_p = fns.get("nl_p") or zero
    return SS(v(fns["u0"]), v(fns["g"]), phi_fn, v(fns["mu_m"]), v(fns["mu_p"]), v(fns["k_m"]),
              v(fns["k_p"]), v(fns["f_m"]), v(fns["f_p"]), v(fns["alpha"]), v(fns["beta"]), nl_m, nl_p)


def per_point(fn, dtype):
    """A product-style callable (r of shape (3, M) -> (M,)) as a reference per-point callable."""

    def f(r):
        x = np.asarray(refjax._raw(r), dtype).reshape(3, 1)
        v = np.asarray(fn(x), dtype).reshape(-1)
        return refjax._wrap(np.asarray(v[0], dtype))

    return f
