"""Host-side API pieces that run without a GPU: mesh construction, model config and
parameter trees, problem definitions."""

import numpy as np
import pytest

from dips_gb300 import mesh, nn, problems


def test_linspace_and_grid_ordering():
    x = mesh.linspace_f32(-1, 1, 32)
    assert x.dtype == np.float32 and x[0] == -1 and x[-1] == 1
    g = mesh.uniform_grid(4)
    assert g.R.shape == (64, 3)
    # 'ij' C-order: z fastest
    assert g.R[1, 2] > g.R[0, 2] and g.R[1, 0] == g.R[0, 0]
    assert g.R_xmin_boundary.shape == (16, 3) and np.all(g.R_xmin_boundary[:, 0] == -1)


def test_model_dict_and_param_tree():
    md = {"model_type": "mlp", "mlp": {"hidden_layers_m": 1, "hidden_dim_m": 1, "activation_m": "jnp.tanh",
                                       "hidden_layers_p": 2, "hidden_dim_p": 10, "activation_p": "jnp.tanh"}}
    fwd, fw = nn.get_model(md, "mlp")
    assert fw == "haiku" and fwd.arch == nn.Arch(1, 1, 2, 10)
    flat = nn.init_params(fwd.arch, 0)
    assert flat.size == nn.n_params(fwd.arch) == 167
    tree = nn.params_to_tree(flat, fwd.arch)
    assert "double_mlp/~mlp_m_fn/linear" in tree and "double_mlp/~mlp_p_fn/linear_2" in tree
    assert tree["double_mlp/~mlp_p_fn/linear_1"]["w"].shape == (10, 10)
    assert tree["preconditioner"] == {}
    back = nn.tree_to_params(tree, fwd.arch).numpy()
    np.testing.assert_array_equal(back, flat)
    with pytest.raises(NotImplementedError):
        nn.arch_from_model_dict({"model_type": "mlp", "mlp": {"activation_m": "nn.celu"}})


def test_problem_callables_numpy_and_torch_agree():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    r = rng.uniform(-1, 1, (3, 500)).astype(np.float32)
    for pr in (problems.sphere_problem(), problems.star_problem()):
        for k in ("phi", "mu_m", "mu_p", "f_m", "f_p", "alpha", "beta", "g"):
            a = np.asarray(pr[k](r), np.float64)
            b = pr[k](torch.as_tensor(r)).double().numpy()
            np.testing.assert_allclose(np.broadcast_to(a, b.shape), b, rtol=1e-5, atol=1e-5)


def test_sphere_beta_is_the_reference_flux_jump_convention():
    pr = problems.sphere_problem()
    # on the sphere: beta = -(mu+ d_n u+ - mu- d_n u-), n = x/|x|
    x = np.array([[0.5], [0.0], [0.0]], np.float32)
    dn_up = 2 * 0.5
    dn_um = np.cos(0.5) * np.cos(0.0) * np.exp(0.0)
    assert np.isclose(pr["beta"](x)[0], -(10.0 * dn_up - 1.0 * dn_um), rtol=1e-6)


def test_nonlinear_operators_are_callables_and_setup_refuses_others():
    torch = pytest.importorskip("torch")
    from dips_gb300 import nonlinear, trainer

    s = nonlinear.Sinh(2.5)
    u = np.linspace(-2, 2, 9).astype(np.float32)
    v = s(u)
    assert v.dtype == np.float32
    np.testing.assert_allclose(v, 2.5 * np.sinh(u), rtol=1e-6)
    np.testing.assert_allclose(s(torch.as_tensor(u)).numpy(), v, rtol=1e-6)
    assert nonlinear.resolve(None).kind == nonlinear.ZERO_KIND and nonlinear.is_zero(None)
    assert nonlinear.resolve(s) is s and not nonlinear.is_zero(s)
    with pytest.raises(NotImplementedError):
        nonlinear.resolve(lambda x: x**3)
    one = lambda r: 1.0  # noqa: E731
    init_fn = trainer.setup(one, one, one, one, one, one, one, one, one, one, one, nonlinear_op_m=s)
    assert callable(init_fn)
    with pytest.raises(NotImplementedError):
        trainer.setup(one, one, one, one, one, one, one, one, one, one, one, nonlinear_op_p=np.cbrt)


def test_optimizer_dict_maps_to_the_step_hyperparameters():
    pytest.importorskip("torch")
    from dips_gb300 import _lib, trainer

    custom = trainer.adam_state_from_dict(10, {"optimizer_name": "custom", "learning_rate": 1e-2,
                                               "sched": {"scheduler_name": "polynomial", "decay_rate": 0.9}}, "cpu")
    assert custom.hp.kind == _lib.OPT_ADAM and custom.hp.schedule == _lib.SCHED_POLYNOMIAL
    assert custom.hp.max_norm == 1.0
    rms = trainer.adam_state_from_dict(10, {"optimizer_name": "rmsprop", "learning_rate": 1e-2}, "cpu")
    assert rms.hp.kind == _lib.OPT_RMSPROP and abs(rms.hp.b2 - 0.9) < 1e-7 and rms.hp.decay_rate == 1.0
    assert rms.hp.max_norm == float("inf")
    adam = trainer.adam_state_from_dict(10, {"optimizer_name": "adam", "learning_rate": 1e-2}, "cpu")
    assert adam.hp.kind == _lib.OPT_ADAM and adam.hp.schedule == _lib.SCHED_EXPONENTIAL and adam.hp.decay_rate == 1.0
    assert trainer.adam_state_from_dict(10, {"optimizer_name": "lbfgs"}, "cpu") is None
    with pytest.raises(ValueError):
        trainer.adam_state_from_dict(10, {"optimizer_name": "custom", "sched": {"scheduler_name": "cosine"}}, "cpu")
    with pytest.raises(ValueError):
        trainer.adam_state_from_dict(10, {"optimizer_name": "sgd"}, "cpu")
