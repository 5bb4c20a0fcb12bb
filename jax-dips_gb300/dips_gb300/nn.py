"""The u-/u+ surrogate networks (mirror of jax_dips/nn/configure.py and nn/mlp/MLP.py).

``get_model(model_dict, model_type)`` returns ``(forward, "haiku")`` like the reference
(nn/configure.py:28-36).  ``forward.init(rng, x, phi_x)`` returns a parameter tree keyed
like haiku's (``double_mlp/~mlp_m_fn/linear``, ``.../linear_1``, ... each with ``w`` and
``b``) and ``forward.apply(params, rng, x, phi_x)`` evaluates u = MLP_p(x) where
phi_x >= 0 else MLP_m(x) (nn/mlp/MLP.py:93-139) with the CUDA kernel.

All device work uses one flat float32 parameter vector (layout in include/dips.h);
the tree holds views into it.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

_TANH_NAMES = {"jnp.tanh", "nn.tanh", "tanh", "torch.tanh", "np.tanh"}


@dataclass(frozen=True)
class Arch:
    m_layers: int = 1
    m_width: int = 1
    p_layers: int = 2
    p_width: int = 10
    # learned preconditioner (nn/preconditioner.py:10-35): tanh layers over the 26 cell
    # coefficients, P = 0.5 + pre_scaling * sigmoid(out); 0 layers = off
    pre_layers: int = 0
    pre_width: int = 0
    pre_scaling: float = 1.0

    def ctype(self):
        return _lib.ArchT(self.m_layers, self.m_width, self.p_layers, self.p_width, self.pre_layers, self.pre_width,
                          self.pre_scaling)

    def net(self, which):
        return (self.m_layers, self.m_width) if which == "m" else (self.p_layers, self.p_width)


def layer_shapes(layers, width, d_in=3):
    shapes, i = [], d_in
    for _ in range(layers):
        shapes.append((i, width))
        i = width
    shapes.append((i, 1))
    return shapes


PRE_IN = 26  # the preconditioner's input: the cell coefficients (geom_pp.py:873-901)


def pre_shapes(arch: Arch):
    return layer_shapes(arch.pre_layers, arch.pre_width, PRE_IN) if arch.pre_layers > 0 else []


def n_params(arch: Arch) -> int:
    nets = sum(a * b + b for w in ("m", "p") for a, b in layer_shapes(*arch.net(w)))
    return nets + sum(a * b + b for a, b in pre_shapes(arch))


def arch_from_model_dict(model_dict: dict) -> Arch:
    mtype = model_dict.get("model_type", "mlp")
    if mtype != "mlp":
        raise NotImplementedError(f"model_type {mtype!r}: only the 'mlp' DoubleMLP runs on the GB300 path")
    mlp = model_dict.get("mlp", {})
    for key in ("activation_m", "activation_p"):
        act = mlp.get(key, "jnp.tanh")
        if act not in _TANH_NAMES:
            raise NotImplementedError(f"{key}={act!r}: only tanh activations have a CUDA kernel")
    pre = model_dict.get("preconditioner") or {}
    pl, pw, ps = 0, 0, 1.0
    if pre.get("enable", False):
        widths = [int(v) for v in pre.get("layer_widths", [])]
        if not widths or len(set(widths)) != 1:
            raise NotImplementedError(f"preconditioner layer_widths {widths}: one width for every layer is supported")
        pl, pw, ps = len(widths), widths[0], float(pre.get("scaling_coeff", 1.0))
    return Arch(int(mlp.get("hidden_layers_m", 1)), int(mlp.get("hidden_dim_m", 1)),
                int(mlp.get("hidden_layers_p", 2)), int(mlp.get("hidden_dim_p", 10)), pl, pw, ps)


def init_params(arch: Arch, seed: int = 0) -> np.ndarray:
    """Haiku-style initial values: hidden w ~ TruncatedNormal(0.1) (MLP.py:65, :70), output
    w ~ TruncatedNormal(1/sqrt(fan_in)) (hk.Linear default), b = 0.  Drawn with numpy."""
    rng = np.random.default_rng(seed)
    parts = []
    for which in ("m", "p"):
        shapes = layer_shapes(*arch.net(which))
        for li, (a, b) in enumerate(shapes):
            std = 0.1 if li < len(shapes) - 1 else 1.0 / np.sqrt(a)
            w = rng.standard_normal((a, b))
            bad = np.abs(w) > 2.0
            while bad.any():
                w[bad] = rng.standard_normal(int(bad.sum()))
                bad = np.abs(w) > 2.0
            # truncated standard normal on [-2, 2] has std 0.87962566...
            parts.append((w * std / 0.87962566103423978).astype(np.float32).ravel())
            parts.append(np.zeros(b, np.float32))
    # preconditioner: flax Dense with glorot_uniform kernels and zero biases (preconditioner.py:18-35)
    for a, b in pre_shapes(arch):
        lim = np.sqrt(6.0 / (a + b))
        parts.append(rng.uniform(-lim, lim, (a, b)).astype(np.float32).ravel())
        parts.append(np.zeros(b, np.float32))
    return np.concatenate(parts).astype(np.float32)


def module_names(arch: Arch):
    names = []
    for which in ("m", "p"):
        L, _ = arch.net(which)
        for li in range(L + 1):
            names.append(f"double_mlp/~mlp_{which}_fn/linear" + ("" if li == 0 else f"_{li}"))
    return names


def params_to_tree(flat, arch: Arch) -> dict:
    """Haiku-shaped tree of views into the flat vector (plus the reference's empty
    ``preconditioner`` entry, trainer.py:244-253)."""
    tree, off = {}, 0
    names = iter(module_names(arch))
    for which in ("m", "p"):
        for a, b in layer_shapes(*arch.net(which)):
            w = flat[off:off + a * b].reshape(a, b)
            off += a * b
            bb = flat[off:off + b]
            off += b
            tree[next(names)] = {"w": w, "b": bb}
    pre = {}
    for li, (a, b) in enumerate(pre_shapes(arch)):
        k = flat[off:off + a * b].reshape(a, b)
        off += a * b
        bb = flat[off:off + b]
        off += b
        pre[f"Dense_{li}"] = {"kernel": k, "bias": bb}
    tree["preconditioner"] = {"params": pre} if pre else {}
    return tree


def tree_to_params(tree: dict, arch: Arch, device=None) -> torch.Tensor:
    parts = []
    for name in module_names(arch):
        parts.append(torch.as_tensor(np.asarray(tree[name]["w"]) if not torch.is_tensor(tree[name]["w"])
                                     else tree[name]["w"]).reshape(-1))
        parts.append(torch.as_tensor(np.asarray(tree[name]["b"]) if not torch.is_tensor(tree[name]["b"])
                                     else tree[name]["b"]).reshape(-1))
    pre = (tree.get("preconditioner") or {}).get("params", {})
    for li in range(len(pre_shapes(arch))):
        for key in ("kernel", "bias"):
            v = pre[f"Dense_{li}"][key]
            parts.append(torch.as_tensor(np.asarray(v) if not torch.is_tensor(v) else v).reshape(-1))
    out = torch.cat([p.to(torch.float32).cpu() for p in parts])
    return out.to(device) if device is not None else out


def mlp_eval(arch: Arch, params: torch.Tensor, pts: torch.Tensor, phi: torch.Tensor, want_grad=False):
    """u (and grad u) at points; the network is chosen by phi >= 0."""
    lib = _lib.load()
    pts = pts.to(torch.float32).contiguous()
    phi = phi.to(torch.float32).contiguous()
    n = pts.shape[0]
    u = torch.empty(n, dtype=torch.float32, device=pts.device)
    g = torch.empty(n, 3, dtype=torch.float32, device=pts.device) if want_grad else None
    _lib.check(lib.dips_mlp_eval(arch.ctype(), _lib.ptr(params), _lib.ptr(pts), _lib.ptr(phi), n, _lib.ptr(u),
                                 _lib.ptr(g), _lib.stream_handle()), "dips_mlp_eval")
    return (u, g) if want_grad else u


class DoubleMLPForward:
    """``hk.transform``-like object with ``init`` and ``apply`` for the DoubleMLP."""

    def __init__(self, arch: Arch):
        self.arch = arch

    def init(self, rng=None, x=None, phi_x=None, seed=None):
        s = int(seed if seed is not None else (rng if isinstance(rng, (int, np.integer)) else 42))
        return params_to_tree(torch.as_tensor(init_params(self.arch, s)), self.arch)

    def apply(self, params, rng, x, phi_x):
        flat = params if torch.is_tensor(params) and params.dim() == 1 else tree_to_params(params, self.arch)
        x = torch.as_tensor(np.asarray(x, np.float32) if not torch.is_tensor(x) else x)
        single = x.dim() == 1
        xs = x.reshape(-1, 3).cuda()
        ph = torch.as_tensor(phi_x, dtype=torch.float32).reshape(-1).cuda().expand(xs.shape[0]).contiguous()
        u = mlp_eval(self.arch, flat.cuda(), xs, ph)
        return u[0] if single else u


def get_model(model_dict: dict, model_type: str = "mlp"):
    """``nn.configure.get_model`` (nn/configure.py:28-50) for the DoubleMLP."""
    if model_type not in ("mlp",):
        raise NotImplementedError(f"model_type {model_type!r} is outside the GB300 path (only 'mlp')")
    md = dict(model_dict)
    md.setdefault("model_type", model_type)
    return DoubleMLPForward(arch_from_model_dict(md)), "haiku"
