"""Residual, loss, adjoint and optimizer entry points over the C ABI, and the
``torch.autograd.Function`` that replaces ``value_and_grad(Trainer.loss)``
(solvers/poisson/trainer.py:783-789, :892-912)."""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .nn import Arch, n_params
from .records import FVLevel


class StepWorkspace:
    """Scratch memory for one batch size and job bound (caller-owned, library-carved)."""

    def __init__(self, arch: Arch, batch: int, max_jobs: int, device="cuda"):
        lib = _lib.load()
        nbytes = int(lib.dips_step_workspace_bytes(arch.ctype(), batch, max_jobs))
        if nbytes == 0:
            raise ValueError("invalid workspace request")
        self.arch, self.batch, self.max_jobs, self.nbytes = arch, batch, max_jobs, nbytes
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device)

    def fits(self, arch, batch, max_jobs):
        return arch == self.arch and batch == self.batch and max_jobs <= self.max_jobs


def _ids_ptr(batch_ids):
    return _lib.ptr(batch_ids) if batch_ids is not None else _lib.c_void_p(0)


def residual_forward(arch: Arch, params: torch.Tensor, level: FVLevel, batch_ids=None, ws: StepWorkspace = None,
                     want_residual=False):
    """Loss (device float64 scalar) and optionally the per-point residuals of a batch."""
    lib = _lib.load()
    B = level.n if batch_ids is None else int(batch_ids.numel())
    if ws is None or not ws.fits(arch, B, level.max_jobs(B)):
        ws = StepWorkspace(arch, B, level.max_jobs(B), params.device)
    loss = torch.empty((), dtype=torch.float64, device=params.device)
    res = torch.empty(B, dtype=torch.float32, device=params.device) if want_residual else None
    _lib.check(lib.dips_residual_fwd(arch.ctype(), _lib.ptr(params), level.desc, _ids_ptr(batch_ids), B,
                                     _lib.ptr(ws.buf), ws.nbytes, _lib.ptr(loss), _lib.ptr(res),
                                     _lib.stream_handle()), "dips_residual_fwd")
    return loss, res, ws


def residual_backward(arch: Arch, params: torch.Tensor, level: FVLevel, batch_ids, ws: StepWorkspace):
    lib = _lib.load()
    B = level.n if batch_ids is None else int(batch_ids.numel())
    grad = torch.empty(n_params(arch), dtype=torch.float32, device=params.device)
    _lib.check(lib.dips_residual_bwd(arch.ctype(), _lib.ptr(params), level.desc, _ids_ptr(batch_ids), B,
                                     _lib.ptr(ws.buf), ws.nbytes, _lib.ptr(grad), _lib.stream_handle()),
               "dips_residual_bwd")
    return grad


def loss_coefficient_derivative(arch: Arch, params: torch.Tensor, level: FVLevel, tangent, batch_ids=None,
                                ws: StepWorkspace = None) -> torch.Tensor:
    """d loss / d theta (device float64 scalar) of the residual_forward loss along the
    coefficient direction of ``tangent`` (``level.coefficient_tangent({...})``), the params
    fixed; e.g. the gradient of the total loss with respect to a constant mu+."""
    lib = _lib.load()
    B = level.n if batch_ids is None else int(batch_ids.numel())
    if ws is None or not ws.fits(arch, B, level.max_jobs(B)):
        ws = StepWorkspace(arch, B, level.max_jobs(B), params.device)
    out = torch.empty((), dtype=torch.float64, device=params.device)
    _lib.check(lib.dips_loss_coeff_tangent(arch.ctype(), _lib.ptr(params), level.desc, tangent.desc,
                                           _ids_ptr(batch_ids), B, _lib.ptr(ws.buf), ws.nbytes, _lib.ptr(out),
                                           _lib.stream_handle()), "dips_loss_coeff_tangent")
    return out


class ResidualLoss(torch.autograd.Function):
    """loss = mean(0.5 * (lhs/diag - rhs/diag)^2) over a batch, differentiable in params."""

    @staticmethod
    def forward(ctx, params, arch, level, batch_ids):
        loss, _, ws = residual_forward(arch, params.detach().contiguous(), level, batch_ids)
        ctx.arch, ctx.level, ctx.batch_ids, ctx.ws = arch, level, batch_ids, ws
        ctx.save_for_backward(params)
        return loss.to(torch.float32)

    @staticmethod
    def backward(ctx, g):
        (params,) = ctx.saved_tensors
        grad = residual_backward(ctx.arch, params.detach().contiguous(), ctx.level, ctx.batch_ids, ctx.ws)
        return grad * g.to(grad.dtype), None, None, None


def residual_loss(params, arch: Arch, level: FVLevel, batch_ids=None):
    return ResidualLoss.apply(params, arch, level, batch_ids)


class AdamState:
    """clip_by_global_norm -> scale_by_adam -> scale_by_schedule(exponential_decay) -> scale(-1)
    (solvers/optimizers.py:33-54); moments and step count live on the device.

    ``kind="rmsprop"`` is optax.rmsprop (b2 is then its decay; mu unused) and
    ``schedule="polynomial"`` optax.polynomial_schedule to 0 over transition_steps (dips_adam_t)."""

    def __init__(self, n: int, lr=1e-3, decay_rate=0.9, transition_steps=1000, max_norm=1.0,
                 b1=0.9, b2=0.999, eps=1e-8, device="cuda", kind="adam", schedule="exponential"):
        self.mu = torch.zeros(n, dtype=torch.float32, device=device)
        self.nu = torch.zeros(n, dtype=torch.float32, device=device)
        self.count = torch.zeros(1, dtype=torch.int64, device=device)
        k = {"adam": _lib.OPT_ADAM, "rmsprop": _lib.OPT_RMSPROP}[kind]
        sc = {"exponential": _lib.SCHED_EXPONENTIAL, "polynomial": _lib.SCHED_POLYNOMIAL}[schedule]
        self.hp = _lib.AdamT(lr, decay_rate, float(transition_steps), max_norm, b1, b2, eps, k, sc)

    def step(self, arch: Arch, params: torch.Tensor, grad: torch.Tensor):
        lib = _lib.load()
        _lib.check(lib.dips_adam_step(arch.ctype(), self.hp, _lib.ptr(params), _lib.ptr(grad), _lib.ptr(self.mu),
                                      _lib.ptr(self.nu), _lib.ptr(self.count), _lib.stream_handle()),
                   "dips_adam_step")


def train_step(arch: Arch, params: torch.Tensor, opt: AdamState, level: FVLevel, batch_ids, ws: StepWorkspace,
               loss_out: torch.Tensor, grad_out=None):
    """One fused step: residual forward, adjoint, gradient reduction and Adam (params in place)."""
    lib = _lib.load()
    B = level.n if batch_ids is None else int(batch_ids.numel())
    _lib.check(lib.dips_train_step(arch.ctype(), opt.hp, _lib.ptr(params), _lib.ptr(opt.mu), _lib.ptr(opt.nu),
                                   _lib.ptr(opt.count), level.desc, _ids_ptr(batch_ids), B, _lib.ptr(ws.buf),
                                   ws.nbytes, _lib.ptr(loss_out), _lib.ptr(grad_out), _lib.stream_handle()),
               "dips_train_step")


def autotune(arch: Arch, params: torch.Tensor, level: FVLevel, batch_ids, ws: StepWorkspace) -> int:
    """Pick the fastest launch configuration of the shape's point kernel on this batch (kept
    process-wide for the current device); returns the warps per CTA chosen (0: nothing to tune).
    Synchronises the stream: call it before capturing a CUDA graph."""
    lib = _lib.load()
    B = level.n if batch_ids is None else int(batch_ids.numel())
    out = ctypes.c_int32(0)
    _lib.check(lib.dips_autotune(arch.ctype(), _lib.ptr(params), level.desc, _ids_ptr(batch_ids), B, _lib.ptr(ws.buf),
                                 ws.nbytes, ctypes.byref(out), _lib.stream_handle()), "dips_autotune")
    return int(out.value)


STEP_PHASES = ("expand", "forward_m", "forward_p", "residual", "fused_m", "fused_p", "loss", "adjoint_m",
               "adjoint_p", "reduce", "adam")


def train_step_profiled(arch: Arch, params: torch.Tensor, opt: AdamState, level: FVLevel, batch_ids,
                        ws: StepWorkspace, loss_out: torch.Tensor, events):
    """train_step with ``len(STEP_PHASES) + 1`` torch.cuda.Events recorded at the phase boundaries
    on the current stream; returns nothing (read the events after a synchronise)."""
    lib = _lib.load()
    B = level.n if batch_ids is None else int(batch_ids.numel())
    for e in events:  # creates the event and marks it recorded for torch; the library records it again
        e.record()
    arr = (ctypes.c_void_p * len(events))(*[e.cuda_event for e in events])
    _lib.check(lib.dips_train_step_profiled(arch.ctype(), opt.hp, _lib.ptr(params), _lib.ptr(opt.mu),
                                            _lib.ptr(opt.nu), _lib.ptr(opt.count), level.desc, _ids_ptr(batch_ids),
                                            B, _lib.ptr(ws.buf), ws.nbytes, _lib.ptr(loss_out), None, arr,
                                            len(events), _lib.stream_handle()),
               "dips_train_step_profiled")


def phase_ms(events):
    """Milliseconds per phase from the events of one train_step_profiled call."""
    return {name: events[i].elapsed_time(events[i + 1]) for i, name in enumerate(STEP_PHASES)}


def batch_ids(n: int, batch: int, epoch: int, batch_index: int, seed: int = 0, out=None, device="cuda"):
    """Ids of minibatch ``batch_index`` of ``epoch``: a seeded permutation of 0..n-1."""
    lib = _lib.load()
    out = out if out is not None else torch.empty(batch, dtype=torch.int32, device=device)
    _lib.check(lib.dips_batch_ids(n, epoch, seed, batch_index, batch, _lib.ptr(out), _lib.stream_handle()),
               "dips_batch_ids")
    return out


class LbfgsResult:
    def __init__(self, params, loss, iterations, evaluations, message, stopped):
        self.params, self.loss, self.iterations, self.evaluations = params, loss, iterations, evaluations
        self.message, self.stopped = message, stopped


def lbfgs_minimize(arch: Arch, params: torch.Tensor, level: FVLevel, batch_ids=None, maxiter: int = 1000,
                   tol: float = 1e-15, callback=None, ws: StepWorkspace = None) -> LbfgsResult:
    """The reference's full-batch L-BFGS path (optimizer_name "lbfgs": trainer.py:204-206 and
    ``solve_jaxopt`` :354-420, i.e. ``jaxopt.ScipyMinimize(method="l-bfgs-b", tol=1e-15,
    maxiter=num_epochs)`` on the loss of one batch): scipy's L-BFGS-B over the flat parameter
    vector in float64, with the loss and its gradient from this library's kernels
    (``dips_residual_fwd`` / ``dips_residual_bwd``).  ``params`` is updated in place.

    ``callback(params, loss)`` runs after every iteration with the current parameters on the
    device and their loss; returning True stops the minimisation (scipy's StopIteration)."""
    from scipy.optimize import minimize

    B = level.n if batch_ids is None else int(batch_ids.numel())
    if ws is None or not ws.fits(arch, B, level.max_jobs(B)):
        ws = StepWorkspace(arch, B, level.max_jobs(B), params.device)
    host = torch.empty(params.numel(), dtype=torch.float32, pin_memory=True)
    counts = {"evals": 0, "iters": 0, "stopped": False, "last": float("nan")}

    def fun(x):
        host.copy_(torch.from_numpy(x.astype(np.float32)))
        params.copy_(host, non_blocking=True)
        loss, _, _ = residual_forward(arch, params, level, batch_ids, ws)
        grad = residual_backward(arch, params, level, batch_ids, ws)
        counts["evals"] += 1
        counts["last"] = float(loss)
        return counts["last"], grad.double().cpu().numpy()

    def cb(xk):
        counts["iters"] += 1
        if callback is not None:
            params.copy_(torch.from_numpy(xk.astype(np.float32)))
            if callback(params, counts["last"]):
                counts["stopped"] = True
                raise StopIteration

    x0 = params.detach().double().cpu().numpy()
    res = minimize(fun, x0, jac=True, method="L-BFGS-B", tol=tol, options={"maxiter": int(maxiter)}, callback=cb)
    params.copy_(torch.from_numpy(np.asarray(res.x, np.float32)))
    return LbfgsResult(params, float(res.fun), counts["iters"], counts["evals"], str(res.message), counts["stopped"])
