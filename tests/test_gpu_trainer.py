"""The reference-facing API end to end on the GPU: trainer.setup -> init_fn -> solve_fn
(solvers/poisson/trainer.py:980-1137) on the sphere problem with the README network
(u- 1x1, u+ 2x10), full batch, and the per-epoch losses checked against the oracle's own
training loop: h = dx * 0.5^(epoch // (E/4)) (data_management.py:319-326), the loss before
each update (trainer.py:783-789), optax's chained Adam (solvers/optimizers.py:33-54).
"""

import numpy as np
import pytest
import torch

import _parity
from dips_gb300 import levelset, mesh, nn, trainer

L = _parity.L
O = _parity.O
F32 = np.float32

pytestmark = pytest.mark.gpu


def _problem():
    return _parity.make_problem("sphere")


def _run_api(n, epochs, lr, pre=None):
    pr = _problem()
    g = mesh.uniform_grid(n)
    phi = lambda r: levelset.perturb(pr["phi"](r))  # noqa: E731  (the caller perturbs, as the examples do)
    init_fn = trainer.setup(pr["u_p"], pr["g"], phi, pr["mu_m"], pr["mu_p"], pr["k_m"], pr["k_p"], pr["f_m"],
                            pr["f_p"], pr["alpha"], pr["beta"])
    opt = {"optimizer_name": "custom", "learning_rate": lr, "sched": {"scheduler_name": "exponential", "decay_rate": 0.9}}
    model = {"model_type": "mlp", "mlp": {"hidden_layers_m": 1, "hidden_dim_m": 1, "activation_m": "jnp.tanh",
                                          "hidden_layers_p": 2, "hidden_dim_p": 10, "activation_p": "jnp.tanh"},
             "preconditioner": pre or {"enable": False}}
    state, solve_fn = init_fn(lvl_gstate=g, tr_gstate=g, eval_gstate=g, num_epochs=epochs, batch_size=n ** 3,
                              optimizer_dict=opt, model_dict=model, print_rate=0, seed=42)
    state, epoch_store, loss_epochs = solve_fn(state)
    return g, pr, state, epoch_store, np.asarray(loss_epochs), solve_fn.trainer


def _oracle_losses(g, pr, epochs, lr, arch, oarch=None):
    phi = O.perturb(np.asarray(pr["phi"](g.R.T), F32))
    prob = L.Problem(phi, g.x, g.y, g.z, pr)
    params = nn.init_params(arch, 42)
    adam = O.ChainedAdam(params.size, lr=lr, decay_rate=0.9)
    q = max(epochs // 4, 1)
    losses, cur, rg = [], None, None
    for e in range(epochs):
        k = e // q
        if k != cur:
            h = np.array([g.dx, g.dy, g.dz], F32) * F32(0.5**k)
            rg = L.ResidualGeometry(prob, g.R, h)
            cur = k
        loss, grad = L.loss_and_grad(params, oarch or L.Arch(1, 1, 2, 10), rg)
        losses.append(float(loss))
        params = adam.update(params, np.asarray(grad, F32))
    return np.array(losses), params


def test_setup_init_solve_tracks_oracle(tmp_path):
    n, epochs, lr = 14, 8, 1e-2
    g, pr, state, epoch_store, losses, tr = _run_api(n, epochs, lr)
    assert list(epoch_store) == list(range(epochs))
    assert losses.shape == (epochs,) and np.isfinite(losses).all()
    ref, p_ref = _oracle_losses(g, pr, epochs, lr, tr.arch)
    np.testing.assert_allclose(losses, ref, rtol=2e-4)
    np.testing.assert_allclose(tr.params.cpu().numpy(), p_ref, rtol=2e-3, atol=2e-5)
    # solution fields on the evaluation grid (trainer.py:1113-1130)
    ne = g.R.shape[0]
    assert tuple(state.solution.shape) in ((ne,), (ne, 1))
    assert tuple(state.grad_solution.shape) == (ne, 3)
    assert torch.isfinite(torch.as_tensor(state.solution)).all()
    # the VTK dump of the evaluation grid holds the same solution (x fastest in the file)
    from dips_gb300 import io

    back = io.read_vts(tr.write_solution_vtk(str(tmp_path / "sol")))
    sol = torch.as_tensor(state.solution).reshape(n, n, n).cpu().numpy()
    np.testing.assert_allclose(back["solution"], sol.transpose(2, 1, 0).reshape(-1), rtol=1e-6, atol=1e-7)


def test_training_reduces_the_solution_error():
    """Longer run: the trained network approaches the exact solution (the learned surrogate
    improves on its initialisation by a wide margin)."""
    n, epochs = 16, 400
    g, pr, state, _, losses, tr = _run_api(n, epochs, 1e-2)
    exact = np.asarray(pr["exact"](g.R.T), F32)
    u = torch.as_tensor(state.solution).reshape(-1).cpu().numpy()
    err = np.max(np.abs(u - exact)) / np.max(np.abs(exact))
    R = torch.as_tensor(g.R, device="cuda")
    u0 = nn.mlp_eval(tr.arch, torch.as_tensor(nn.init_params(tr.arch, 42), device="cuda"), R, tr.ls(R))
    err0 = np.max(np.abs(u0.cpu().numpy() - exact)) / np.max(np.abs(exact))
    msg = f"loss {losses[0]:.3e} -> {losses[-1]:.3e}, rel L-inf error {err0:.3f} -> {err:.3f}"
    print(msg)
    assert losses[-1] < 0.2 * losses[0], msg
    assert err < 0.5 * err0, msg


def test_learned_preconditioner_through_the_api():
    """model_dict["preconditioner"] = {enable, layer_widths, scaling_coeff} (trainer.py:229-243):
    the preconditioner's parameters are trained with the networks and the per-epoch losses follow
    the oracle's loop with the same preconditioner."""
    n, epochs, lr = 12, 6, 1e-2
    pre = {"enable": True, "layer_widths": [16, 16], "scaling_coeff": 1.0}
    g, pr, state, _, losses, tr = _run_api(n, epochs, lr, pre)
    assert (tr.arch.pre_layers, tr.arch.pre_width) == (2, 16)
    tree = nn.params_to_tree(tr.params.cpu(), tr.arch)
    assert sorted(tree["preconditioner"]["params"]) == ["Dense_0", "Dense_1", "Dense_2"]
    ref, _ = _oracle_losses(g, pr, epochs, lr, tr.arch, L.Arch(1, 1, 2, 10, 2, 16, 1.0))
    # Adam's first steps move each parameter by about +-lr by the sign of its gradient; a
    # gradient component of the preconditioner near zero can take the other sign under another
    # summation order, after which the trajectories part by O(lr) in that parameter.  The first
    # epochs are held tightly, the rest to the trajectory's spread (the per-step loss and
    # gradient parity of the preconditioner is in test_gpu_parity.py).
    np.testing.assert_allclose(losses[:2], ref[:2], rtol=1e-4)
    np.testing.assert_allclose(losses, ref, rtol=3e-2)
