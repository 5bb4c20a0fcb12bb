"""``setup -> init_fn -> solve_fn``: the reference's NBM Poisson API (mirror of
jax_dips/solvers/poisson/trainer.py:980-1137) running on the GB300 kernels.

Differences from the reference, all on purpose:

* Coefficient callables receive coordinates as an array ``r`` of shape (3, M) (a torch
  tensor on the GPU) instead of one point; ``x, y, z = r`` and ``r[0]`` work unchanged.
* phi is sampled on ``lvl_gstate`` and interpolated trilinearly
  (domain/interpolate.py:906-1021); the reference evaluates the callable directly
  (discretization.py:90).
* The training step is one CUDA graph: batch ids from the device step counter, residual
  forward, adjoint, gradient reduction, chained Adam.
* ``model_dict["preconditioner"]`` may be absent (the reference requires it,
  trainer.py:229); an enabled one (uniform ``layer_widths``) is trained with the networks.
* ``optimizer_name == "lbfgs"`` runs scipy's L-BFGS-B on the GPU loss and gradient instead of
  jaxopt (solve_jaxopt, trainer.py:354-420).
* Nonlinear operators are ``None`` or one of ``dips_gb300.nonlinear``'s kinds.
"""

from __future__ import annotations

import dataclasses
import logging
import os
import pickle
import re
from typing import Callable

import numpy as np
import torch

from . import _lib, dp, levelset, nn, nonlinear, ops
from .mesh import GridState
from .records import FVLevel, eval_callable

logger = logging.getLogger(__name__)
F32 = np.float32


@dataclasses.dataclass
class PoissonSimStateFn:
    """The 13 callables (solvers/simulation_states.py:11-25)."""

    u_0_fn: Callable
    dir_bc_fn: Callable
    phi_fn: Callable
    mu_m_fn: Callable
    mu_p_fn: Callable
    k_m_fn: Callable
    k_p_fn: Callable
    f_m_fn: Callable
    f_p_fn: Callable
    alpha_fn: Callable
    beta_fn: Callable
    nonlinear_op_m: Callable
    nonlinear_op_p: Callable


@dataclasses.dataclass
class PoissonSimState:
    """The 13 arrays (solvers/simulation_states.py:58-80)."""

    phi: object
    solution: object
    dirichlet_bc: object
    mu_m: object
    mu_p: object
    k_m: object
    k_p: object
    f_m: object
    f_p: object
    alpha: object
    beta: object
    grad_solution: object
    grad_normal_solution: object


DEFAULT_OPTIMIZER = {"optimizer_name": "custom", "learning_rate": 1e-3,
                     "sched": {"scheduler_name": "exponential", "decay_rate": 0.9}}
DEFAULT_MODEL = {"name": None, "model_type": "mlp",
                 "mlp": {"hidden_layers_m": 1, "hidden_dim_m": 1, "activation_m": "jnp.tanh",
                         "hidden_layers_p": 2, "hidden_dim_p": 10, "activation_p": "jnp.tanh"}}


def adam_state_from_dict(n_params, optimizer_dict, device):
    """``get_optimizer`` (solvers/optimizers.py:57-97) for the Adam variants."""
    name = optimizer_dict.get("optimizer_name", "custom")
    lr = float(optimizer_dict.get("learning_rate", 1e-3))
    sched = optimizer_dict.get("sched", {}) or {}
    if name == "custom":
        sname = sched.get("scheduler_name", "exponential")
        if sname not in ("exponential", "polynomial"):  # get_scheduler (optimizers.py:13-30)
            raise ValueError(f"Unknown scheduler: {sname}")
        return ops.AdamState(n_params, lr=lr, decay_rate=float(sched.get("decay_rate", 0.96)), transition_steps=1000,
                             max_norm=1.0, device=device, schedule=sname)
    if name == "adam":  # optax.adam: no clipping, constant rate
        return ops.AdamState(n_params, lr=lr, decay_rate=1.0, transition_steps=1000, max_norm=float("inf"),
                             device=device)
    if name == "rmsprop":  # optax.rmsprop(lr): decay 0.9, eps 1e-8, no clipping, constant rate
        return ops.AdamState(n_params, lr=lr, decay_rate=1.0, transition_steps=1000, max_norm=float("inf"), b2=0.9,
                             eps=1e-8, device=device, kind="rmsprop")
    if name == "lbfgs":  # Trainer.solve runs scipy's L-BFGS-B instead (solve_jaxopt, trainer.py:354-420)
        return None
    raise ValueError(f"Unknown optimizer: {name}")


_TUNED = set()


def _to_numpy(tree):
    """Nested dict of tensors -> nested dict of numpy arrays (checkpoint contents)."""
    if isinstance(tree, dict):
        return {k: _to_numpy(v) for k, v in tree.items()}
    return np.asarray(tree.detach().cpu() if torch.is_tensor(tree) else tree)


def _levels(num_epochs):
    q = max(num_epochs // 4, 1)
    return (num_epochs - 1) // q + 1 if num_epochs > 0 else 1


class Trainer:
    """NBM training on one GPU (Trainer, solvers/poisson/trainer.py:81-977)."""

    def __init__(self, lvl_gstate: GridState, tr_gstate: GridState, eval_gstate: GridState, sim_state_fn,
                 num_epochs=1000, batch_size=131072, optimizer_dict=None, model_dict=None, batching="sequential",
                 seed=0, checkpoint_dir=None, restart=False, restart_checkpoint_dir=None, use_graph=True,
                 device="cuda", multi_gpu=False, checkpoint_interval=None):
        if not torch.cuda.is_available():
            raise RuntimeError("dips_gb300 runs on a CUDA GPU; none is available")
        _lib.load()
        self.device = device
        self.fn = sim_state_fn
        self.lvl_gstate, self.tr_gstate, self.eval_gstate = lvl_gstate, tr_gstate, eval_gstate
        model_dict = dict(model_dict or DEFAULT_MODEL)
        self.arch = nn.arch_from_model_dict(model_dict)  # includes the learned preconditioner if enabled
        if not _lib.load().dips_arch_supported(self.arch.ctype()):
            raise NotImplementedError(_lib.load().dips_last_error().decode())
        self.num_epochs = int(num_epochs)
        self.seed = seed
        self.batching = batching
        self.use_graph = use_graph
        self.checkpoint_dir = checkpoint_dir
        self.checkpoint_interval = int(checkpoint_interval or 0)
        # ---- level set on the level-set grid (samples of the user's phi callable)
        self.ls = levelset.LevelSetGrid.from_callable(lvl_gstate, sim_state_fn.phi_fn, device)
        # ---- training points, batches (DatasetDict, data/data_management.py:79-159)
        pts = np.asarray(tr_gstate.R, F32)
        n = pts.shape[0]
        bs = min(int(batch_size), n)
        self.multi_gpu = bool(multi_gpu)
        self.rank, self.world = 0, 1
        if self.multi_gpu:
            # one process per GPU: this rank trains on its DatasetDict device run and the
            # gradients are summed across ranks every step (trainer.py:716-834)
            if not torch.distributed.is_initialized():
                raise RuntimeError("multi_gpu needs torch.distributed initialised, one process per GPU")
            self.rank, self.world = torch.distributed.get_rank(), torch.distributed.get_world_size()
            pts, bs, nb = dp.device_points(pts, self.world * int(batch_size), self.rank, self.world,
                                           lambda c: self._padding_points(np.asarray(tr_gstate.R, F32), c))
            self.batching = "sequential"
            self.use_graph = False
        elif batching == "sequential":
            nb, extra = n // bs, n % bs
            if extra:
                pad = self._padding_points(pts, bs - extra)
                pts = np.concatenate([pts, pad]).astype(F32)
                nb += 1
        elif batching == "uniform":
            nb = n // bs
        else:
            raise ValueError("batching must be 'sequential' or 'uniform'")
        self.n_points, self.batch, self.n_batches = n, bs, nb
        self.points = torch.as_tensor(pts, device=device)
        self.h0 = np.array([tr_gstate.dx, tr_gstate.dy, tr_gstate.dz], F32)
        self.n_levels = _levels(self.num_epochs)
        # ---- params and optimizer
        P = nn.n_params(self.arch)
        self.params = torch.as_tensor(nn.init_params(self.arch, 42 if seed is None else seed), device=device)
        self.optimizer_name = (optimizer_dict or DEFAULT_OPTIMIZER).get("optimizer_name", "custom")
        self.opt = adam_state_from_dict(P, optimizer_dict or DEFAULT_OPTIMIZER, device)
        if self.opt is None:  # L-BFGS: no optimizer state on the device; the checkpoint keeps a zero one
            self.opt = ops.AdamState(P, device=device)
        self.epoch_start = 0
        if restart:
            self._restore(restart_checkpoint_dir)
        self.loss_dev = torch.zeros((), dtype=torch.float64, device=device)
        self.loss_epoch_acc = torch.zeros((), dtype=torch.float64, device=device)
        self.ids = torch.empty(self.batch, dtype=torch.int32, device=device)
        self._level_cache = {}

    # ------------------------------------------------------------------ data
    @staticmethod
    def _padding_points(pts, count, seed=0):
        """Random points rescaled to the data range (generate_random_points_like,
        data_management.py:70-76); drawn with numpy instead of jax's PRNGKey(0)."""
        rng = np.random.default_rng(seed)
        dR = rng.standard_normal((count, 3))
        lo, hi = float(pts.min()), float(pts.max())
        return (lo + (hi - lo) * (dR - dR.min()) / (dR.max() - dR.min())).astype(F32)

    def level(self, k) -> FVLevel:
        if k not in self._level_cache:
            self._level_cache.clear()
            h = self.h0 * F32(0.5**k)
            fns = {"mu_m": self.fn.mu_m_fn, "mu_p": self.fn.mu_p_fn, "k_m": self.fn.k_m_fn, "k_p": self.fn.k_p_fn,
                   "f_m": self.fn.f_m_fn, "f_p": self.fn.f_p_fn, "alpha": self.fn.alpha_fn, "beta": self.fn.beta_fn,
                   "g": self.fn.dir_bc_fn, "nl_m": self.fn.nonlinear_op_m, "nl_p": self.fn.nonlinear_op_p}
            # the learned preconditioner reads the 26 cell coefficients of each point
            self._level_cache[k] = FVLevel(self.ls, fns, self.points, h, keep_geometry=self.arch.pre_layers > 0)
        return self._level_cache[k]

    # ------------------------------------------------------------------ step
    def _step(self, lvl, ws):
        lib = _lib.load()
        mode = 0 if self.batching == "sequential" else 1
        n_ids = self.points.shape[0] if mode == 0 else self.n_points
        _lib.check(lib.dips_batch_ids_device(n_ids, self.batch, self.n_batches, self.seed or 0, mode,
                                             _lib.ptr(self.opt.count), _lib.ptr(self.ids), _lib.stream_handle()),
                   "dips_batch_ids_device")
        if self.multi_gpu:  # update_multi_gpu (trainer.py:824-834): psum of grads and loss, then Adam
            loss, _, _ = ops.residual_forward(self.arch, self.params, lvl, self.ids, ws)
            grad = ops.residual_backward(self.arch, self.params, lvl, self.ids, ws)
            dp.allreduce_sum_(grad, loss)
            self.opt.step(self.arch, self.params, grad)
            self.loss_epoch_acc += loss
            return
        ops.train_step(self.arch, self.params, self.opt, lvl, self.ids, ws, self.loss_dev)
        self.loss_epoch_acc += self.loss_dev

    def _make_runner(self, lvl):
        ws = ops.StepWorkspace(self.arch, self.batch, lvl.max_jobs(self.batch, distinct=True), self.device)
        a = self.arch
        key = (a.m_layers, a.m_width, a.p_layers, a.p_width, str(self.device))
        if key not in _TUNED:  # launch-configuration autotuner, once per shape and device, before any capture
            ids = ops.batch_ids(self.points.shape[0], self.batch, epoch=0, batch_index=0, seed=99, device=self.device)
            ops.autotune(self.arch, self.params, lvl, ids, ws)
            _TUNED.add(key)
        if not self.use_graph:
            return lambda: self._step(lvl, ws), ws
        # warm up outside the capture (sets kernel attributes), then undo its effect
        saved = [t.clone() for t in (self.params, self.opt.mu, self.opt.nu, self.opt.count, self.loss_epoch_acc)]
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._step(lvl, ws)
        torch.cuda.current_stream().wait_stream(s)
        for t, v in zip((self.params, self.opt.mu, self.opt.nu, self.opt.count, self.loss_epoch_acc), saved):
            t.copy_(v)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._step(lvl, ws)
        return g.replay, ws

    def solve_lbfgs(self, print_rate=1, callback=None):
        """``solve_jaxopt`` (trainer.py:354-420): scipy's L-BFGS-B (tol 1e-15, at most num_epochs
        iterations) on the loss of the first batch at the training spacing h = dx, the loss and
        gradient from the GPU kernels.  Returns the iteration numbers and the loss after each."""
        lvl = self.level(0)
        ids = torch.arange(self.batch, dtype=torch.int32, device=self.device)  # DatasetDict batch 0
        losses = []

        def cb(p, loss):
            losses.append(loss)
            if print_rate and (len(losses) - 1) % print_rate == 0:
                logger.info("lbfgs iteration %d loss %.6e", len(losses) - 1, losses[-1])
            return bool(callback(len(losses) - 1, losses[-1])) if callback is not None else False

        res = ops.lbfgs_minimize(self.arch, self.params, lvl, ids, maxiter=self.num_epochs, tol=1e-15, callback=cb)
        self.lbfgs_result = res
        self.epoch_store = np.arange(len(losses))
        self.loss_epochs = np.asarray(losses)
        if self.checkpoint_dir and self.rank == 0:
            self.save_checkpoint(self.checkpoint_dir, len(losses))
        return self.epoch_store, self.loss_epochs

    def solve(self, print_rate=1, callback=None):
        """Epoch loop (single_GPU_train, trainer.py:501-591); with optimizer_name "lbfgs" the
        reference's solve_jaxopt instead (trainer.py:204-206)."""
        if self.optimizer_name == "lbfgs":
            return self.solve_lbfgs(print_rate, callback)
        loss_epochs = np.zeros(self.num_epochs - self.epoch_start)
        q = max(self.num_epochs // 4, 1)
        cur, run = None, None
        for epoch in range(self.epoch_start, self.num_epochs):
            k = epoch // q  # alternate_res_sequentially (data_management.py:319-326)
            if k != cur:
                lvl = self.level(k)
                run, _ = self._make_runner(lvl)
                cur = k
            self.loss_epoch_acc.zero_()
            for _ in range(self.n_batches):
                run()
            loss_epochs[epoch - self.epoch_start] = float(self.loss_epoch_acc) / self.n_batches
            if print_rate and (epoch % print_rate == 0):
                logger.info("epoch %d loss %.6e", epoch, loss_epochs[epoch - self.epoch_start])
            if callback is not None:
                callback(epoch, loss_epochs[epoch - self.epoch_start])
            self._interval_checkpoint(epoch)
        self.epoch_store = np.arange(self.epoch_start, self.num_epochs)
        self.loss_epochs = loss_epochs
        if self.checkpoint_dir and self.rank == 0:  # the ranks hold the same state: one writer
            self.save_checkpoint(self.checkpoint_dir, self.num_epochs)
        return self.epoch_store, loss_epochs

    # ------------------------------------------------------------------ evaluation
    def evaluate_solution_and_gradients(self, gstate: GridState):
        """u, grad u and d_n u on a grid (trainer.py:929-977): d_n u = n . grad u with n the
        normalised central difference of the interpolated phi at spacing (dx, dy, dz)
        (``normal_point_fn``, discretization.py:199-218)."""
        R = torch.as_tensor(gstate.R, device=self.device)
        phi = self.ls(R)
        u, gu = nn.mlp_eval(self.arch, self.params, R, phi, want_grad=True)
        h = (gstate.dx, gstate.dy, gstate.dz)
        d = []
        for a in range(3):
            rp, rm = R.clone(), R.clone()
            rp[:, a] += float(h[a])
            rm[:, a] -= float(h[a])
            d.append((self.ls(rp) - self.ls(rm)) / (2.0 * float(h[a])))
        nrm = torch.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
        nx, ny, nz = d[0] / nrm, d[1] / nrm, d[2] / nrm
        gn = nx * gu[:, 0] + ny * gu[:, 1] + nz * gu[:, 2]
        return u, gu, gn

    # ------------------------------------------------------------------ checkpoints
    def write_solution_vtk(self, filename="results/solution", gstate: GridState = None):
        """u, grad u, d_n u and phi on a grid as a VTK structured grid (the reference's
        write_vtk_manual, utils/io.py:80-88)."""
        from . import io

        gstate = gstate or self.eval_gstate
        u, gu, gn = self.evaluate_solution_and_gradients(gstate)
        R = torch.as_tensor(gstate.R, device=self.device)
        shape = (gstate.x.shape[0], gstate.y.shape[0], gstate.z.shape[0])
        fields = {"solution": u.reshape(shape), "grad_solution": gu.reshape(shape + (3,)),
                  "grad_normal_solution": gn.reshape(shape), "phi": self.ls(R).reshape(shape)}
        return io.write_vtk_manual(gstate, fields, filename)

    def _interval_checkpoint(self, epoch):
        """multi_GPU_train's checkpoints (trainer.py:769-777): after every checkpoint_interval-th
        epoch, written by rank 0.  The reference's single-GPU loop saves at the end only
        (trainer.py:470-477), and so does this one."""
        if (self.multi_gpu and self.rank == 0 and self.checkpoint_dir and self.checkpoint_interval > 0
                and (epoch + 1) % self.checkpoint_interval == 0):
            return self.save_checkpoint(self.checkpoint_dir, epoch + 1)
        return None

    def save_checkpoint(self, checkpoint_dir, epoch):
        """pickle of {opt_state, params, epoch, batch_size, resolution} (trainer.py:340-351).

        ``params`` is the haiku parameter tree, as the reference stores it.  ``opt_state`` is
        this library's flat layout {mu, nu, count} (flat float32 moments in the parameter
        vector's order), not optax's ScaleByAdamState tree: a reference checkpoint's params load
        here, its optimizer state does not, and the reverse holds as well."""
        os.makedirs(checkpoint_dir, exist_ok=True)
        state = {
            "opt_state": {"mu": self.opt.mu.cpu().numpy(), "nu": self.opt.nu.cpu().numpy(),
                          "count": int(self.opt.count.item())},
            "params": _to_numpy(nn.params_to_tree(self.params, self.arch)),
            "epoch": int(epoch),
            "batch_size": int(self.batch),
            "resolution": f"{self.h0[0]}, {self.h0[1]}, {self.h0[2]}",
        }
        path = os.path.join(checkpoint_dir, "checkpoint_" + str(epoch))
        with open(path, "wb") as f:
            pickle.dump(state, f)
        return path

    def _restore(self, checkpoint_dir):
        """fetch_checkpoint (trainer.py:326-338): the highest-numbered checkpoint.  The reference
        picks max() by string and then resets the epoch to 0 (trainer.py:261); here the epoch
        number is compared numerically and training resumes at the stored epoch."""
        if not checkpoint_dir or not os.path.isdir(checkpoint_dir):
            return
        # only names this trainer writes ("checkpoint_<epoch>"): a stray "checkpoint_100.tmp" or a
        # backup copy beside them is skipped, not parsed
        cks = [p for p in os.listdir(checkpoint_dir) if re.fullmatch(r"checkpoint_(\d+)", p)]
        if not cks:
            return
        best = max(cks, key=lambda p: int(p.split("_")[-1]))
        with open(os.path.join(checkpoint_dir, best), "rb") as f:
            state = pickle.load(f)
        stored = int(state.get("batch_size", self.batch))
        if stored != self.batch:
            # the reference resumes with the checkpoint's batch size (trainer.py:215); the batches
            # of this trainer are laid out already, so a different size is refused, not adopted
            raise ValueError(f"checkpoint {best} was written with batch_size {stored}, this trainer uses "
                             f"{self.batch}; construct it with batch_size={stored} to resume")
        self.params.copy_(nn.tree_to_params(state["params"], self.arch, self.device))
        self.opt.mu.copy_(torch.as_tensor(state["opt_state"]["mu"], device=self.device))
        self.opt.nu.copy_(torch.as_tensor(state["opt_state"]["nu"], device=self.device))
        self.opt.count.fill_(int(state["opt_state"]["count"]))
        self.epoch_start = min(int(state["epoch"]), self.num_epochs)


def setup(initial_value_fn, dirichlet_bc_fn, lvl_set_fn, mu_m_fn_, mu_p_fn_, k_m_fn_, k_p_fn_, f_m_fn_, f_p_fn_,
          alpha_fn_, beta_fn_, nonlinear_op_m=None, nonlinear_op_p=None):
    """``trainer.setup`` (trainer.py:980-1137).

    ``nonlinear_op_m/p``: None (zero, the reference's default) or an operator of
    ``dips_gb300.nonlinear`` (``Sinh(c)``: N(u) = c sinh(u)); any other callable raises
    NotImplementedError, since the residual kernel evaluates the operator on the GPU."""
    fn = PoissonSimStateFn(initial_value_fn, dirichlet_bc_fn, lvl_set_fn, mu_m_fn_, mu_p_fn_, k_m_fn_, k_p_fn_,
                           f_m_fn_, f_p_fn_, alpha_fn_, beta_fn_, nonlinear.resolve(nonlinear_op_m),
                           nonlinear.resolve(nonlinear_op_p))

    def init_fn(lvl_gstate: GridState = None, tr_gstate: GridState = None, eval_gstate: GridState = None,
                num_epochs: int = 1000, batch_size: int = 131072, algorithm: int = 0,
                mgrad_over_pgrad_scalefactor: int = 1, multi_gpu: bool = False, checkpoint_interval: int = 1000,
                checkpoint_dir: str = "./checkpoints", results_dir: str = "./", loss_plot_name: str = "solver_loss",
                optimizer_dict: dict = None, model_dict: dict = None, restart: bool = False,
                restart_checkpoint_dir: str = "./checkpoints", print_rate: int = 1, batching: str = "sequential",
                seed: int = 42, use_graph: bool = True):
        """``init_fn`` (trainer.py:1035-1136): the initial state on ``eval_gstate`` and ``solve_fn``.

        Accepted for the reference's signature and without effect here: ``results_dir`` and
        ``loss_plot_name`` (the reference's matplotlib loss plot; ``solve_fn`` returns the losses)
        and ``mgrad_over_pgrad_scalefactor``, which has no effect in the reference either (its one
        use is in ``Trainer.__update``, trainer.py:792-815, which nothing calls)."""
        if algorithm != 0:
            raise NotImplementedError("algorithm 1 (network extrapolation) is unimplemented in the reference too")
        R = torch.as_tensor(eval_gstate.R, device="cuda")
        ev = lambda f: eval_callable(f, R)  # noqa: E731
        state = PoissonSimState(ev(lvl_set_fn), ev(initial_value_fn), ev(dirichlet_bc_fn), ev(mu_m_fn_),
                                ev(mu_p_fn_), ev(k_m_fn_), ev(k_p_fn_), ev(f_m_fn_), ev(f_p_fn_), ev(alpha_fn_),
                                ev(beta_fn_), None, None)

        def solve_fn(sim_state: PoissonSimState):
            tr = Trainer(lvl_gstate, tr_gstate, eval_gstate, fn, num_epochs=num_epochs, batch_size=batch_size,
                         optimizer_dict=optimizer_dict, model_dict=model_dict, batching=batching, seed=seed,
                         checkpoint_dir=checkpoint_dir, restart=restart, restart_checkpoint_dir=restart_checkpoint_dir,
                         use_graph=use_graph, multi_gpu=multi_gpu, checkpoint_interval=checkpoint_interval)
            epoch_store, loss_epochs = tr.solve(print_rate=print_rate)
            u, gu, gn = tr.evaluate_solution_and_gradients(eval_gstate)
            new = dataclasses.replace(sim_state, solution=u, grad_solution=gu, grad_normal_solution=gn)
            solve_fn.trainer = tr
            return new, epoch_store, loss_epochs

        return state, solve_fn

    return init_fn
