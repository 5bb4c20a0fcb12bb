"""The numpy stand-in for jax (oracle/refjax.py) keeps the jax semantics that the reference's
residual code depends on.  The golden vectors of tests/golden/ref_*.npz come from the
reference's own files run on it, so each rule it restates is checked here on small cases whose
jax results follow from jax 0.4.13's documented behaviour:

* x64 off: values canonicalised to float32 / int32; Python scalars are weakly typed;
* ``.at[].set`` / ``.at[].add`` return new arrays;
* out-of-range integer indices of a gather are clamped;
* ``linalg.det``: closed forms for 2x2 and 3x3;
* ``linalg.pinv``: singular values at or below 10 max(m, n) eps sigma_max are dropped;
* ``argsort`` is stable with NaN last; ``isclose`` follows |a - b| <= atol + rtol |b|;
* ``vmap`` maps over the leading axis, ``lax.cond`` picks a branch, ``jit`` is the identity.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


@pytest.fixture(scope="module")
def jx():
    import refjax

    refjax.install(x64=False)
    jax = sys.modules["jax"]
    yield jax, jax.numpy, refjax
    refjax.set_x64(False)


def test_dtype_canonicalisation_and_weak_scalars(jx):
    jax, jnp, _ = jx
    assert jnp.array(1.0).dtype == np.float32
    assert jnp.arange(3).dtype == np.int32
    assert jnp.asarray(np.zeros(2, np.float64)).dtype == np.float32
    a = jnp.array([1.0, 2.0])
    assert (a * 2.5).dtype == np.float32  # a weak Python float keeps float32
    i = jnp.array([1, 2])
    assert (i + 1).dtype == np.int32
    assert (i * 0.5).dtype == np.float32  # int array with a Python float: the default float


def test_at_updates_return_copies(jx):
    _, jnp, _ = jx
    a = jnp.zeros(4)
    b = a.at[1].set(3.0)
    c = b.at[1].add(2.0)
    np.testing.assert_array_equal(np.asarray(a), [0, 0, 0, 0])
    np.testing.assert_array_equal(np.asarray(b), [0, 3, 0, 0])
    np.testing.assert_array_equal(np.asarray(c), [0, 5, 0, 0])


def test_out_of_range_gather_indices_are_clamped(jx):
    _, jnp, _ = jx
    a = jnp.array([10.0, 20.0, 30.0])
    assert float(a[jnp.array(5)]) == 30.0
    np.testing.assert_array_equal(np.asarray(a[jnp.array([-7, 1, 9])]), [10.0, 20.0, 30.0])


def test_det_closed_forms(jx):
    _, jnp, _ = jx
    rng = np.random.default_rng(0)
    m2 = rng.standard_normal((2, 2)).astype(np.float32)
    m3 = rng.standard_normal((3, 3)).astype(np.float32)
    d2 = float(jnp.linalg.det(jnp.asarray(m2)))
    d3 = float(jnp.linalg.det(jnp.asarray(m3)))
    np.testing.assert_allclose(d2, np.linalg.det(m2.astype(np.float64)), rtol=1e-5)
    np.testing.assert_allclose(d3, np.linalg.det(m3.astype(np.float64)), rtol=1e-5)


def test_pinv_cutoff(jx):
    _, jnp, _ = jx
    # singular values 1 and 1e-9: the second is below 10 * 3 * eps_f32 * 1 and is dropped
    u, _ = np.linalg.qr(np.random.default_rng(1).standard_normal((3, 3)))
    m = (u[:, :2] * np.array([1.0, 1e-9])) @ u[:, :2].T
    p = np.asarray(jnp.linalg.pinv(jnp.asarray(m.astype(np.float32))), np.float64)
    proj = u[:, :1] @ u[:, :1].T  # pinv of the rank-1 part
    np.testing.assert_allclose(p, proj, atol=1e-5)
    # a well-conditioned matrix is inverted
    q = np.diag([2.0, 4.0, 8.0]).astype(np.float32)
    np.testing.assert_allclose(np.asarray(jnp.linalg.pinv(jnp.asarray(q))), np.diag([0.5, 0.25, 0.125]), rtol=1e-6)


def test_argsort_stable_nan_last_and_isclose(jx):
    _, jnp, _ = jx
    v = jnp.array([2.0, np.nan, 1.0, 2.0, -0.0, 0.0])
    np.testing.assert_array_equal(np.asarray(jnp.argsort(v)), [4, 5, 2, 0, 3, 1])
    a = jnp.array([1.0, 1.0 + 1e-6, np.inf, np.nan])
    b = jnp.array([1.0, 1.0, np.inf, np.nan])
    np.testing.assert_array_equal(np.asarray(jnp.isclose(a, b)), [True, True, True, False])


def test_vmap_cond_and_jit(jx):
    jax, jnp, _ = jx

    def f(x):
        return jax.lax.cond(x[0] > 0, lambda y: y * 2.0, lambda y: y - 1.0, x)

    xs = jnp.array([[1.0, 2.0], [-1.0, 3.0]])
    out = np.asarray(jax.vmap(f)(xs))
    np.testing.assert_array_equal(out, [[2.0, 4.0], [-2.0, 2.0]])
    g = jax.jit(lambda x: x + 1.0)
    np.testing.assert_array_equal(np.asarray(g(jnp.array([1.0]))), [2.0])
