"""A numpy stand-in for the small part of ``jax`` that the reference's hot-path modules use.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module.  It exists so that
the reference's own, unmodified source files

* ``jax_dips/solvers/poisson/discretization.py``
* ``jax_dips/geometry/geometric_integrations_per_point.py``
* ``jax_dips/geometry/level_set.py``
* ``jax_dips/domain/interpolate.py``
* ``jax_dips/domain/mesh.py``, ``jax_dips/solvers/simulation_states.py``,
  ``jax_dips/_jaxmd_modules/{util,dataclasses}.py``
* ``tests/confs/experiment_configs.py`` (the reference's manufactured problems)

can be imported and run on a machine without jax/jaxlib (jax 0.4.13 is the pinned version,
``requirements.txt:1``).  Their outputs become golden vectors generated by the reference's
code (``tests/golden/make_reference_golden.py``).

What is restated, and how (jax 0.4.13 semantics, x64 disabled unless ``install(x64=True)``):

* arrays: ``JArray``, an immutable-by-convention ``numpy.ndarray`` subclass with ``.at[].set``
  and ``.at[].add`` returning copies, indexing that returns 0-d arrays and clamps
  out-of-range integer indices as jax's gathers do, and augmented assignment that rebinds
  instead of writing in place;
* dtypes: every value is canonicalised to 32-bit types (float32/int32) with x64 off, as jax
  does; the promotion of a binary operation follows jax's lattice with weakly typed Python
  scalars (bool < int < float; a Python float with an int array gives the default float);
* ``jit``: identity; ``vmap``: a Python loop over the mapped axis, outputs stacked;
  ``lax.cond``: the selected branch (the unselected branch of jax's batched ``cond`` only
  feeds a ``select``, so values are the same);
* ``jnp.linalg.det``: jax's closed forms for 2x2 and 3x3 matrices, LU otherwise;
* ``@``, ``jnp.dot``, ``jnp.matmul``: each output accumulated over the contracted index in
  order, without fused multiply-adds (XLA's CPU loop for small operands);
* ``jnp.linalg.pinv``: jax's rule -- SVD, singular values at or below
  ``10 * max(m, n) * eps * sigma_max`` dropped;
* ``jnp.argsort``/``jnp.sort``: stable, NaN last, -0 == +0 (jax's total-order comparator);
* ``jnp.isclose``: ``|a - b| <= atol + rtol |b|`` in the operands' dtype, with jax's
  handling of infinities and NaN;
* ``grad``/``jvp``: fourth-order central differences evaluated in float64, then cast.  Only
  the reference's problem definitions use them (the flux jump beta needs grad of phi and of
  the exact solutions); no function on the residual path differentiates.

One difference that remains: XLA may fuse element-wise float32 operations differently from
the operation-by-operation numpy evaluation here (for instance with fused multiply-adds).
No discrete decision of the residual path depends on such a last-bit difference on the
parity cases (the fixtures record the crossing flags and the GPU tests compare them exactly).
"""

from __future__ import annotations

import functools
import math
import sys
import types

import numpy as np

_STATE = {"x64": False}


def _float():
    return np.float64 if _STATE["x64"] else np.float32


def _int():
    return np.int64 if _STATE["x64"] else np.int32


def canon_dtype(dt):
    """jax's dtype canonicalisation: 64-bit types become 32-bit with x64 off."""
    if dt is None:
        return None
    if dt is float:
        return np.dtype(_float())
    if dt is int:
        return np.dtype(_int())
    if dt is bool:
        return np.dtype(np.bool_)
    dt = np.dtype(dt)
    if not _STATE["x64"]:
        if dt == np.float64:
            return np.dtype(np.float32)
        if dt == np.int64:
            return np.dtype(np.int32)
        if dt == np.uint64:
            return np.dtype(np.uint32)
        if dt == np.complex128:
            return np.dtype(np.complex64)
    return dt


def _default_dtype_of(x):
    """dtype jnp.asarray gives a Python scalar or a nested list."""
    a = np.asarray(x)
    if a.dtype.kind == "f":
        return canon_dtype(a.dtype) if isinstance(x, (np.ndarray, np.generic)) else np.dtype(_float())
    if a.dtype.kind in "iu":
        return canon_dtype(a.dtype) if isinstance(x, (np.ndarray, np.generic)) else np.dtype(_int())
    return a.dtype


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, _unwrap_index(idx))


class _AtIndex:
    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = idx

    def set(self, v):
        out = np.array(self.arr, copy=True).view(np.ndarray)
        out[self.idx] = np.asarray(_raw(v)).astype(out.dtype)
        return _wrap(out)

    def add(self, v):
        out = np.array(self.arr, copy=True).view(np.ndarray)
        np.add.at(out, self.idx, np.asarray(_raw(v)).astype(out.dtype))
        return _wrap(out)

    def get(self):
        return self.arr[self.idx]


def _raw(x):
    if isinstance(x, JArray):
        return x.view(np.ndarray)
    return x


def _unwrap_index(idx):
    if isinstance(idx, tuple):
        return tuple(_unwrap_index(i) for i in idx)
    if isinstance(idx, JArray):
        a = idx.view(np.ndarray)
        if a.ndim == 0 and a.dtype.kind in "iu":
            return int(a)
        return a
    return idx


def _clamp_index(idx, shape):
    """jax's gather semantics for integer indices: a negative index counts from the end, then an
    out-of-range index is clamped into [0, size - 1] (numpy would raise).  Applied to integer and
    integer-array entries of an index without an Ellipsis; slices and None pass unchanged."""
    t = idx if isinstance(idx, tuple) else (idx,)
    if any(e is Ellipsis for e in t):
        return idx
    out, axis = [], 0
    for e in t:
        if e is None:
            out.append(e)
            continue
        if axis < len(shape) and (isinstance(e, (int, np.integer)) and not isinstance(e, bool)):
            n = shape[axis]
            e = int(e)
            e = e + n if e < 0 else e
            out.append(min(max(e, 0), n - 1))
        elif axis < len(shape) and isinstance(e, np.ndarray) and e.dtype.kind in "iu":
            n = shape[axis]
            out.append(np.clip(np.where(e < 0, e + n, e), 0, n - 1))
        else:
            out.append(e)
        axis += 1
    return tuple(out) if isinstance(idx, tuple) else out[0]


def _wrap(r):
    """Any numpy result -> JArray with a canonical dtype."""
    if isinstance(r, tuple):
        return tuple(_wrap(x) for x in r)
    if isinstance(r, list):
        return [_wrap(x) for x in r]
    if isinstance(r, (np.ndarray, np.generic)):
        a = np.asarray(r)
        dt = canon_dtype(a.dtype)
        if dt != a.dtype:
            a = a.astype(dt)
        return a.view(JArray)
    if isinstance(r, (bool, int, float)):
        return r
    return r


# --------------------------------------------------------------------------------------------
# type promotion (jax's lattice restricted to bool < int < float, with weak Python scalars)
# --------------------------------------------------------------------------------------------
def _result_dtype(args):
    strong = []
    weak_float = weak_int = False
    for a in args:
        if isinstance(a, bool):
            continue
        if isinstance(a, int):
            weak_int = True
        elif isinstance(a, float):
            weak_float = True
        elif isinstance(a, (np.ndarray, np.generic)):
            strong.append(np.asarray(a).dtype)
    floats = [d for d in strong if d.kind == "f"]
    ints = [d for d in strong if d.kind in "iu"]
    if floats:
        return canon_dtype(max(floats, key=lambda d: d.itemsize))
    if weak_float:
        return np.dtype(_float())
    if ints:
        return canon_dtype(max(ints, key=lambda d: d.itemsize))
    if weak_int:
        return np.dtype(_int())
    if strong:
        return strong[0]
    return None


_NO_CAST = {"isnan", "isinf", "isfinite", "signbit", "logical_not", "invert"}


class JArray(np.ndarray):
    """numpy array with jax's value semantics for the operations the reference uses."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _At(self)

    def __getitem__(self, idx):
        raw = self.view(np.ndarray)
        r = np.ndarray.__getitem__(raw, _clamp_index(_unwrap_index(idx), raw.shape))
        return _wrap(r)

    def __setitem__(self, idx, v):  # jax arrays are immutable
        raise TypeError("JArray is immutable; use .at[].set()")

    def __iter__(self):
        for i in range(self.shape[0]):
            yield self[i]

    def astype(self, dtype, **kw):
        return _wrap(self.view(np.ndarray).astype(canon_dtype(dtype)))

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        if kwargs.get("out") is not None:
            raise TypeError("in-place update of a JArray")
        raw = [_raw(x) for x in inputs]
        if ufunc is np.matmul and method == "__call__":
            return seq_matmul(*raw)
        if method == "__call__" and ufunc.__name__ not in _NO_CAST and ufunc.nin >= 1:
            dt = _result_dtype(raw)
            if dt is not None and ufunc.__name__ not in ("left_shift", "right_shift"):
                raw = [np.asarray(x).astype(dt) if not isinstance(x, np.ndarray) or x.dtype != dt else x
                       for x in raw]
        r = getattr(ufunc, method)(*raw, **kwargs)
        return _wrap(r)

    # augmented assignment rebinds, as with immutable jax arrays
    def __iadd__(self, o):
        return self.__add__(o)

    def __isub__(self, o):
        return self.__sub__(o)

    def __imul__(self, o):
        return self.__mul__(o)

    def __itruediv__(self, o):
        return self.__truediv__(o)

    def __ipow__(self, o):
        return self.__pow__(o)

    def __imatmul__(self, o):
        return self.__matmul__(o)

    def __iand__(self, o):
        return self.__and__(o)

    def __ior__(self, o):
        return self.__or__(o)

    def sum(self, axis=None, dtype=None, keepdims=False, **kw):
        return _reduce(np.sum, self, axis, dtype, keepdims)

    def mean(self, axis=None, dtype=None, keepdims=False, **kw):
        a = self.view(np.ndarray)
        r = np.mean(a, axis=axis, dtype=canon_dtype(dtype) or (a.dtype if a.dtype.kind == "f" else _float()),
                    keepdims=keepdims)
        return _wrap(r)

    def min(self, axis=None, keepdims=False, **kw):
        return _wrap(np.min(self.view(np.ndarray), axis=axis, keepdims=keepdims))

    def max(self, axis=None, keepdims=False, **kw):
        return _wrap(np.max(self.view(np.ndarray), axis=axis, keepdims=keepdims))

    def reshape(self, *shape, **kw):
        if not shape:  # jax: x.reshape() is x.reshape(())
            shape = ((),)
        return _wrap(self.view(np.ndarray).reshape(*shape, **kw))

    def flatten(self):
        return _wrap(self.view(np.ndarray).flatten())

    def squeeze(self, axis=None):
        return _wrap(self.view(np.ndarray).squeeze(axis))

    def __bool__(self):
        return bool(self.view(np.ndarray))

    def __index__(self):
        return int(self.view(np.ndarray))

    def __hash__(self):
        raise TypeError("unhashable JArray")


def seq_matmul(a, b):
    """``a @ b`` (or ``jnp.dot`` of 1-d/2-d operands) with each output accumulated over the
    contracted index in order, one rounding per multiply and per add (no fused multiply-add):
    the loop XLA's CPU dot emitter generates for small operands.  BLAS may reorder or fuse."""
    a = np.asarray(a)
    b = np.asarray(b)
    dt = _result_dtype([a, b])
    a = a.astype(dt)
    b = b.astype(dt)
    va, vb = a.ndim == 1, b.ndim == 1
    A = a[None, :] if va else a
    B = b[:, None] if vb else b
    k = A.shape[-1]
    if B.shape[-2] != k:
        raise ValueError(f"matmul shapes {a.shape} {b.shape}")
    acc = A[..., :, 0:1] * B[..., 0:1, :]
    for j in range(1, k):
        acc = (acc + A[..., :, j:j + 1] * B[..., j:j + 1, :]).astype(dt)
    if va:
        acc = acc[..., 0, :]
    if vb:
        acc = acc[..., 0]
    return _wrap(acc.astype(dt))


def _reduce(fn, a, axis, dtype, keepdims):
    a = np.asarray(_raw(a))
    if dtype is None and a.dtype.kind in "biu":
        dtype = _int()
    return _wrap(fn(a, axis=axis, dtype=canon_dtype(dtype), keepdims=keepdims))


# --------------------------------------------------------------------------------------------
# jax.numpy
# --------------------------------------------------------------------------------------------
def _np_namespace():
    m = types.ModuleType("jax.numpy")
    m.__refjax__ = True

    def asarray(x, dtype=None):
        if isinstance(x, JArray) and dtype is None:
            return x
        if dtype is None:
            dtype = _default_dtype_of(_raw_nested(x))
        return _wrap(np.asarray(_raw_nested(x), dtype=canon_dtype(dtype)))

    def array(x, dtype=None, copy=True, **kw):
        return asarray(x, dtype)

    m.asarray = asarray
    m.array = array
    m.ndarray = np.ndarray
    m.newaxis = None
    m.pi = np.pi
    m.inf = np.inf
    m.nan = np.nan
    m.index_exp = np.index_exp
    m.float32 = _ScalarType(np.float32)
    m.float64 = _ScalarType(np.float64)
    m.int32 = _ScalarType(np.int32)
    m.int64 = _ScalarType(np.int64)
    m.int16 = _ScalarType(np.int16)
    m.bool_ = np.bool_
    m.dtype = np.dtype
    m.finfo = np.finfo
    m.iinfo = np.iinfo

    def zeros(shape, dtype=None):
        return _wrap(np.zeros(shape, canon_dtype(dtype) or _float()))

    def ones(shape, dtype=None):
        return _wrap(np.ones(shape, canon_dtype(dtype) or _float()))

    def zeros_like(a, dtype=None):
        return _wrap(np.zeros_like(np.asarray(_raw(a)), dtype=canon_dtype(dtype)))

    def ones_like(a, dtype=None):
        return _wrap(np.ones_like(np.asarray(_raw(a)), dtype=canon_dtype(dtype)))

    def eye(n, m_=None, k=0, dtype=None):
        return _wrap(np.eye(n, m_, k, dtype=canon_dtype(dtype) or _float()))

    def arange(*args, dtype=None):
        if dtype is None:
            dtype = _float() if any(isinstance(a, float) for a in args) else _int()
        return _wrap(np.arange(*[_raw(a) for a in args], dtype=canon_dtype(dtype)))

    def linspace(start, stop, num=50, endpoint=True, dtype=None):
        """jax's linspace: start*(1-t) + stop*t with t = iota/div, the end point exact."""
        dt = canon_dtype(dtype) or np.dtype(_float())
        start = np.asarray(start, dt)
        stop = np.asarray(stop, dt)
        div = (num - 1) if endpoint else num
        if num == 1:
            return _wrap(np.array([start], dt))
        t = (np.arange(num if not endpoint else num - 1, dtype=dt) / dt.type(div)).astype(dt)
        out = (start * (dt.type(1.0) - t) + stop * t).astype(dt)
        if endpoint:
            out = np.concatenate([out, np.array([stop], dt)])
        return _wrap(out)

    def where(cond, x=None, y=None):
        if x is None and y is None:
            return _wrap(np.nonzero(np.asarray(_raw(cond))))
        xr, yr = _raw(x), _raw(y)
        dt = _result_dtype([xr, yr])
        xa = np.asarray(xr).astype(dt)
        ya = np.asarray(yr).astype(dt)
        return _wrap(np.where(np.asarray(_raw(cond)).astype(bool), xa, ya))

    def _unary(fn, floating=True):
        def f(x, *a, **k):
            xr = np.asarray(_raw(x)) if not isinstance(x, (int, float, bool)) else x
            if isinstance(xr, np.ndarray):
                if floating and xr.dtype.kind in "biu":
                    xr = xr.astype(_float())
            elif floating:
                xr = np.asarray(xr, _float())
            else:
                xr = np.asarray(xr, _default_dtype_of(xr))
            with np.errstate(all="ignore"):
                return _wrap(fn(xr, *a, **k))

        return f

    for name in ("sqrt", "exp", "log", "sin", "cos", "tan", "tanh", "arctan", "arcsin", "arccos", "log1p",
                 "expm1", "floor", "ceil", "rint", "sinh", "cosh", "log2", "exp2", "round", "trunc"):
        setattr(m, name, _unary(getattr(np, name)))
    for name in ("abs", "sign", "negative", "square", "absolute"):
        setattr(m, name, _unary(getattr(np, name), floating=False))

    def _binary(fn):
        def f(a, b):
            ar, br = _raw(a), _raw(b)
            dt = _result_dtype([ar, br])
            with np.errstate(all="ignore"):
                return _wrap(fn(np.asarray(ar).astype(dt), np.asarray(br).astype(dt)))

        return f

    for name in ("add", "subtract", "multiply", "divide", "true_divide", "maximum", "minimum", "power",
                 "arctan2", "hypot", "less", "greater", "equal", "not_equal", "less_equal", "greater_equal",
                 "logical_and", "logical_or", "mod", "fmod"):
        setattr(m, name, _binary(getattr(np, name)))

    def nan_to_num(x, copy=True, nan=0.0, posinf=None, neginf=None):
        a = np.asarray(_raw(x))
        if a.dtype.kind not in "fc":
            return _wrap(a)
        fi = np.finfo(a.dtype)
        return _wrap(np.nan_to_num(a, nan=nan, posinf=fi.max if posinf is None else posinf,
                                   neginf=fi.min if neginf is None else neginf))

    def isclose(a, b, rtol=1e-05, atol=1e-08, equal_nan=False):
        ar, br = _raw(a), _raw(b)
        dt = _result_dtype([ar, br])
        a_ = np.asarray(ar).astype(dt)
        b_ = np.asarray(br).astype(dt)
        if dt.kind != "f":
            return _wrap(a_ == b_)
        rt = np.asarray(_raw(rtol)).astype(dt)
        at_ = np.asarray(_raw(atol)).astype(dt)
        with np.errstate(all="ignore"):
            out = np.abs(a_ - b_) <= (at_ + rt * np.abs(b_))
            a_inf, b_inf = np.isinf(a_), np.isinf(b_)
            any_inf = a_inf | b_inf
            both_inf = a_inf & b_inf
            out = np.where(any_inf, both_inf & (a_ == b_), out)
            a_nan, b_nan = np.isnan(a_), np.isnan(b_)
            any_nan = a_nan | b_nan
            out = np.where(any_nan, (a_nan & b_nan) if equal_nan else False, out)
        return _wrap(out)

    def argsort(a, axis=-1, kind="stable", order=None):
        x = np.asarray(_raw(a))
        if x.dtype.kind == "f":
            x = np.where(x == 0, np.zeros_like(x), x)  # -0 == +0
        return _wrap(np.argsort(x, axis=axis, kind="stable").astype(_int()))

    def sort(a, axis=-1, kind="stable", order=None):
        x = np.asarray(_raw(a))
        idx = np.argsort(np.where(x == 0, np.zeros_like(x), x) if x.dtype.kind == "f" else x, axis=axis,
                         kind="stable")
        return _wrap(np.take_along_axis(x, idx, axis=axis))

    def count_nonzero(a, axis=None, keepdims=False):
        return _wrap(np.asarray(np.count_nonzero(np.asarray(_raw(a)), axis=axis, keepdims=keepdims),
                                dtype=_int()))

    def dot(a, b, precision=None):
        ar, br = np.asarray(_raw(a)), np.asarray(_raw(b))
        if ar.ndim == 0 or br.ndim == 0:
            return _wrap(np.multiply(*[x.astype(_result_dtype([ar, br])) for x in (ar, br)]))
        return seq_matmul(ar, br)

    def matmul(a, b, precision=None):
        return seq_matmul(_raw(a), _raw(b))

    def diag(v, k=0):
        return _wrap(np.diag(np.asarray(_raw(v)), k))

    def _seq(fn):
        def f(arrs, *a, **k):
            raws = [np.asarray(_raw(x)) for x in arrs]
            dt = _result_dtype(raws)
            return _wrap(fn([x.astype(dt) for x in raws], *a, **k))

        return f

    m.concatenate = _seq(np.concatenate)
    m.stack = _seq(np.stack)
    m.column_stack = _seq(np.column_stack)
    m.hstack = _seq(np.hstack)
    m.vstack = _seq(np.vstack)

    def split(a, indices_or_sections, axis=0):
        return [_wrap(x) for x in np.split(np.asarray(_raw(a)), indices_or_sections, axis=axis)]

    def meshgrid(*xs, indexing="xy", **kw):
        return [_wrap(x) for x in np.meshgrid(*[np.asarray(_raw(x)) for x in xs], indexing=indexing)]

    def expand_dims(a, axis):
        return _wrap(np.expand_dims(np.asarray(_raw(a)), axis))

    def reshape(a, shape, order="C"):
        return _wrap(np.reshape(np.asarray(_raw(a)), shape, order=order))

    def sum(a, axis=None, dtype=None, keepdims=False, **kw):
        return _reduce(np.sum, a, axis, dtype, keepdims)

    def mean(a, axis=None, dtype=None, keepdims=False, **kw):
        return asarray(a).mean(axis=axis, dtype=dtype, keepdims=keepdims)

    def amin(a, axis=None, keepdims=False, **kw):
        return _wrap(np.min(np.asarray(_raw(a)), axis=axis, keepdims=keepdims))

    def amax(a, axis=None, keepdims=False, **kw):
        return _wrap(np.max(np.asarray(_raw(a)), axis=axis, keepdims=keepdims))

    def clip(a, a_min=None, a_max=None):
        return _wrap(np.clip(np.asarray(_raw(a)), a_min, a_max))

    def squeeze(a, axis=None):
        return _wrap(np.squeeze(np.asarray(_raw(a)), axis))

    def swapaxes(a, x, y):
        return _wrap(np.swapaxes(np.asarray(_raw(a)), x, y))

    def transpose(a, axes=None):
        return _wrap(np.transpose(np.asarray(_raw(a)), axes))

    def ravel(a):
        return _wrap(np.ravel(np.asarray(_raw(a))))

    def any_(a, axis=None):
        return _wrap(np.any(np.asarray(_raw(a)), axis=axis))

    def all_(a, axis=None):
        return _wrap(np.all(np.asarray(_raw(a)), axis=axis))

    def isnan(a):
        return _wrap(np.isnan(np.asarray(_raw(a))))

    def isinf(a):
        return _wrap(np.isinf(np.asarray(_raw(a))))

    def isfinite(a):
        return _wrap(np.isfinite(np.asarray(_raw(a))))

    for name, fn in dict(nan_to_num=nan_to_num, isclose=isclose, argsort=argsort, sort=sort,
                         count_nonzero=count_nonzero, dot=dot, matmul=matmul, diag=diag, split=split,
                         meshgrid=meshgrid, expand_dims=expand_dims, reshape=reshape, sum=sum, mean=mean,
                         min=amin, max=amax, amin=amin, amax=amax, clip=clip, squeeze=squeeze, swapaxes=swapaxes,
                         transpose=transpose, ravel=ravel, any=any_, all=all_, isnan=isnan, isinf=isinf,
                         isfinite=isfinite, where=where, zeros=zeros, ones=ones, zeros_like=zeros_like,
                         ones_like=ones_like, eye=eye, arange=arange, linspace=linspace).items():
        setattr(m, name, fn)

    # ---- jax.numpy.linalg
    lin = types.ModuleType("jax.numpy.linalg")

    def det(a):
        """jax's det: closed forms for 2x2 and 3x3 (left-to-right products and sums), LU otherwise."""
        x = np.asarray(_raw(a))
        if x.shape[-2:] == (2, 2):
            return _wrap(x[..., 0, 0] * x[..., 1, 1] - x[..., 0, 1] * x[..., 1, 0])
        if x.shape[-2:] == (3, 3):
            return _wrap(
                x[..., 0, 0] * x[..., 1, 1] * x[..., 2, 2]
                + x[..., 0, 1] * x[..., 1, 2] * x[..., 2, 0]
                + x[..., 0, 2] * x[..., 1, 0] * x[..., 2, 1]
                - x[..., 0, 2] * x[..., 1, 1] * x[..., 2, 0]
                - x[..., 0, 0] * x[..., 1, 2] * x[..., 2, 1]
                - x[..., 0, 1] * x[..., 1, 0] * x[..., 2, 2]
            )
        return _wrap(np.linalg.det(x).astype(x.dtype))

    def pinv(a, rcond=None):
        """jax's pinv: u, s, vh = svd(a); s <= rcond * s_max -> dropped; vh^T diag(1/s) u^T."""
        x = np.asarray(_raw(a))
        dt = x.dtype
        if rcond is None:
            rcond = 10.0 * max(x.shape[-2:]) * np.finfo(dt).eps
        rcond = np.asarray(rcond, dt)
        u, s, vh = np.linalg.svd(x, full_matrices=False)
        u, s, vh = u.astype(dt), s.astype(dt), vh.astype(dt)
        cutoff = rcond * s[..., 0:1]
        with np.errstate(divide="ignore"):
            s = np.where(s > cutoff, s, np.inf).astype(dt)
            res = np.matmul(np.swapaxes(vh, -1, -2), np.swapaxes(u, -1, -2) / s[..., :, None])
        return _wrap(res.astype(dt))

    def norm(a, ord=None, axis=None, keepdims=False):
        return _wrap(np.linalg.norm(np.asarray(_raw(a)), ord=ord, axis=axis, keepdims=keepdims))

    def inv(a):
        x = np.asarray(_raw(a))
        return _wrap(np.linalg.inv(x).astype(x.dtype))

    def svd(a, full_matrices=True, compute_uv=True):
        x = np.asarray(_raw(a))
        return _wrap(np.linalg.svd(x, full_matrices=full_matrices, compute_uv=compute_uv))

    lin.det = det
    lin.pinv = pinv
    lin.norm = norm
    lin.inv = inv
    lin.svd = svd
    m.linalg = lin

    def __getattr__(name):  # anything else: the numpy function with canonical outputs
        fn = getattr(np, name)
        if callable(fn):
            @functools.wraps(fn)
            def g(*a, **k):
                return _wrap(fn(*[_raw(x) for x in a], **{kk: _raw(v) for kk, v in k.items()}))

            return g
        return fn

    m.__getattr__ = __getattr__
    return m, lin


def _raw_nested(x):
    if isinstance(x, (list, tuple)):
        return [_raw_nested(v) for v in x]
    return _raw(x)


class _ScalarType:
    """``jnp.float32`` etc.: callable (casts, canonicalised) and usable as a dtype."""

    def __init__(self, t):
        self.t = t
        self.dtype = np.dtype(t)

    def __call__(self, x):
        return _wrap(np.asarray(_raw(x)).astype(canon_dtype(self.t)))

    def __eq__(self, other):
        try:
            return np.dtype(other) == self.dtype
        except TypeError:
            return False

    def __hash__(self):
        return hash(self.dtype)

    def __repr__(self):
        return f"jnp.{self.dtype.name}"

    # numpy accepts objects with a .dtype attribute as dtype specifiers


# --------------------------------------------------------------------------------------------
# transformations
# --------------------------------------------------------------------------------------------
def jit(fun=None, *, static_argnums=None, static_argnames=None, backend=None, donate_argnums=None, **kw):
    if fun is None:
        return lambda f: f
    return fun


def _axis_size(args, in_axes):
    for a, ax in zip(args, in_axes):
        if ax is not None:
            return np.shape(_raw(a))[ax]
    raise ValueError("vmap: no mapped argument")


def _take(a, ax, i):
    if ax is None:
        return a
    if isinstance(a, (tuple, list)):
        return type(a)(_take(v, ax, i) for v in a)
    x = np.asarray(_raw(a))
    return _wrap(np.take(x, i, axis=ax))


def _stack(outs):
    o0 = outs[0]
    if isinstance(o0, tuple):
        return tuple(_stack([o[k] for o in outs]) for k in range(len(o0)))
    if isinstance(o0, list):
        return [_stack([o[k] for o in outs]) for k in range(len(o0))]
    if isinstance(o0, dict):
        return {k: _stack([o[k] for o in outs]) for k in o0}
    raws = [_raw(o) for o in outs]
    dt = _result_dtype(raws) if any(isinstance(r, (np.ndarray, np.generic)) for r in raws) else None
    if dt is None:
        dt = _default_dtype_of(raws[0])
    return _wrap(np.stack([np.asarray(r).astype(dt) for r in raws]))


def vmap(fun, in_axes=0, out_axes=0, **kw):
    """Python loop over the mapped axis.  A function marked ``__refjax_batched__`` (the test
    harness's own network) is called once with the whole batch instead."""

    @functools.wraps(fun) if hasattr(fun, "__name__") else (lambda f: f)
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        target = fun.func if isinstance(fun, functools.partial) else fun
        if getattr(target, "__refjax_batched__", False) and all(ax in (0, None) for ax in axes):
            return fun(*args)
        n = _axis_size(args, axes)
        outs = [fun(*[_take(a, ax, i) for a, ax in zip(args, axes)]) for i in range(n)]
        if n == 0:
            raise ValueError("vmap over an empty axis")
        return _stack(outs)

    return mapped


def _fd_grad(f, x, argnums=0):
    """Fourth-order central differences of f at x, evaluated in float64."""
    old = _STATE["x64"]
    _STATE["x64"] = True
    try:
        x64 = np.asarray(_raw(x), np.float64)
        g = np.zeros_like(x64)
        flat = g.reshape(-1)
        for i in range(x64.size):
            h = 1e-4 * max(1.0, abs(float(x64.reshape(-1)[i])))
            vals = []
            for s in (-2, -1, 1, 2):
                xp = x64.copy().reshape(-1)
                xp[i] += s * h
                vals.append(float(np.asarray(_raw(f(_wrap(xp.reshape(x64.shape)))))))
            flat[i] = (vals[0] - 8 * vals[1] + 8 * vals[2] - vals[3]) / (12 * h)
    finally:
        _STATE["x64"] = old
    return _wrap(g.astype(canon_dtype(np.asarray(_raw(x)).dtype)))


def grad(fun, argnums=0, **kw):
    def g(*args):
        def f1(x):
            a = list(args)
            a[argnums] = x
            return fun(*a)

        return _fd_grad(f1, args[argnums])

    return g


def jvp(fun, primals, tangents):
    x = primals[0]
    t = np.asarray(_raw(tangents[0]), np.float64)
    old = _STATE["x64"]
    _STATE["x64"] = True
    try:
        x64 = np.asarray(_raw(x), np.float64)
        h = 1e-4
        vals = [np.asarray(_raw(fun(_wrap(x64 + s * h * t))), np.float64) for s in (-2, -1, 1, 2)]
        d = (vals[0] - 8 * vals[1] + 8 * vals[2] - vals[3]) / (12 * h)
    finally:
        _STATE["x64"] = old
    return fun(x), _wrap(d.astype(_float()))


# --------------------------------------------------------------------------------------------
# lax
# --------------------------------------------------------------------------------------------
def _lax_module():
    lax = types.ModuleType("jax.lax")

    def cond(pred, true_fun, false_fun, *operands, **kw):
        return true_fun(*operands) if bool(np.asarray(_raw(pred))) else false_fun(*operands)

    def fori_loop(lower, upper, body, init):
        val = init
        for i in range(int(lower), int(upper)):
            val = body(np.int32(i), val)
        return val

    def select(pred, on_true, on_false):
        return _wrap(np.where(np.asarray(_raw(pred)), _raw(on_true), _raw(on_false)))

    lax.cond = cond
    lax.fori_loop = fori_loop
    lax.select = select

    def _missing(name):
        def f(*a, **k):
            raise NotImplementedError(f"jax.lax.{name} is not provided by the stand-in")

        return f

    for name in ("conv_general_dilated", "conv_dimension_numbers", "scan", "while_loop"):
        setattr(lax, name, _missing(name))
    return lax


class _Config:
    def update(self, name, value):
        if name == "jax_enable_x64":
            _STATE["x64"] = bool(value)

    def __getattr__(self, name):
        if name == "jax_enable_x64":
            return _STATE["x64"]
        return False


def install(x64=False):
    """Register the stand-in as ``jax`` (and its submodules) in ``sys.modules``.

    Call this only in a process that runs the reference's code (a fixture generator or a
    subprocess of a test); the product never sees it."""
    _STATE["x64"] = bool(x64)
    jax = types.ModuleType("jax")
    jnp, lin = _np_namespace()
    lax = _lax_module()
    cfg = _Config()
    jax.numpy = jnp
    jax.lax = lax
    jax.config = cfg
    jax.jit = jit
    jax.vmap = vmap
    jax.grad = grad
    jax.jvp = jvp
    jax.Array = np.ndarray
    jax.__refjax__ = True

    tu = types.ModuleType("jax.tree_util")
    tu.register_pytree_node = lambda *a, **k: None
    tu.tree_map = lambda f, *trees: _tree_map(f, *trees)
    tu.tree_leaves = lambda t: _tree_leaves(t)
    jax.tree_util = tu

    lib = types.ModuleType("jax.lib")
    xb = types.ModuleType("jax.lib.xla_bridge")
    xb.get_backend = lambda *a: types.SimpleNamespace(platform="cpu")
    lib.xla_bridge = xb
    jax.lib = lib

    src = types.ModuleType("jax._src")
    api = types.ModuleType("jax._src.api")
    api.vmap = vmap
    api.jit = jit
    src.api = api
    jax._src = src

    rnd = types.ModuleType("jax.random")

    def _no_random(*a, **k):
        raise NotImplementedError("jax.random is not provided by the stand-in")

    rnd.PRNGKey = _no_random
    rnd.normal = _no_random
    rnd.split = _no_random
    rnd.multivariate_normal = _no_random
    jax.random = rnd

    mods = {
        "jax": jax,
        "jax.numpy": jnp,
        "jax.numpy.linalg": lin,
        "jax.lax": lax,
        "jax.tree_util": tu,
        "jax.lib": lib,
        "jax.lib.xla_bridge": xb,
        "jax._src": src,
        "jax._src.api": api,
        "jax.random": rnd,
    }
    for k, v in mods.items():
        existing = sys.modules.get(k)
        if existing is not None and not getattr(existing, "__refjax__", False) and k == "jax":
            raise RuntimeError("a real jax is already imported; the stand-in would shadow it")
        sys.modules[k] = v
    return jax


def set_x64(flag: bool):
    _STATE["x64"] = bool(flag)


def _tree_map(f, *trees):
    t0 = trees[0]
    if isinstance(t0, dict):
        return {k: _tree_map(f, *[t[k] for t in trees]) for k in t0}
    if isinstance(t0, (list, tuple)):
        return type(t0)(_tree_map(f, *[t[i] for t in trees]) for i in range(len(t0)))
    return f(*trees)


def _tree_leaves(t):
    if isinstance(t, dict):
        out = []
        for k in t:
            out += _tree_leaves(t[k])
        return out
    if isinstance(t, (list, tuple)):
        out = []
        for v in t:
            out += _tree_leaves(v)
        return out
    return [t]


__all__ = ["install", "set_x64", "JArray", "canon_dtype", "math"]
