"""Nonlinear operators N-(u), N+(u) of the residual (the reference's ``nonlinear_op_m/p``).

The reference adds N-(u-) V- + N+(u+) V+ to the left-hand side at every interior point
(solvers/poisson/discretization.py:369), with u-/u+ the extrapolated pair at the point itself
(``get_u_mp_by_regression_at_point_fn``, :426-519) and V-/V+ the cell's volumes on either side.
``trainer.setup`` takes arbitrary jax callables for them (trainer.py:992-1017) and defaults both
to zero.  Here the GPU evaluates the operator inside the residual kernel, so it is one of a
fixed set of kinds that the kernel knows:

* ``Zero()``     N(u) = 0 (the reference's default)
* ``Sinh(c)``    N(u) = c sinh(u) (the nonlinear Poisson-Boltzmann term of the reference's
  biomolecule example, ``examples/biomolecules/coefficients.py:126-132``: kappa^2 sinh(u))

Each is also a plain callable on numpy arrays and torch tensors, so the same object serves the
oracle and the reference-side harness.  ``resolve`` turns ``setup``'s arguments into one of
these and refuses any other callable: the GPU path cannot run an arbitrary Python function per
point.
"""

from __future__ import annotations

import numpy as np

ZERO_KIND = 0  # DIPS_NL_ZERO
SINH_KIND = 1  # DIPS_NL_SINH


class Zero:
    kind = ZERO_KIND
    c = 0.0

    def __call__(self, u):
        return u * 0.0

    def __repr__(self):
        return "Zero()"


class Sinh:
    """N(u) = c sinh(u)."""

    kind = SINH_KIND

    def __init__(self, c: float):
        self.c = float(c)

    def __call__(self, u):
        try:
            import torch

            if isinstance(u, torch.Tensor):
                return self.c * torch.sinh(u)
        except ImportError:  # pragma: no cover
            pass
        # numpy arrays and their subclasses keep their type and float32 stays float32
        return self.c * np.sinh(u)

    def __repr__(self):
        return f"Sinh({self.c!r})"


def resolve(op):
    """``setup``'s nonlinear_op argument as one of the kinds above (None: zero)."""
    if op is None:
        return Zero()
    if isinstance(op, (Zero, Sinh)):
        return op
    raise NotImplementedError(
        "nonlinear operators on the GB300 path are dips_gb300.nonlinear.Zero() or Sinh(c) "
        f"(N(u) = c sinh(u)); got {op!r}")


def is_zero(op) -> bool:
    return op is None or isinstance(op, Zero) or (isinstance(op, Sinh) and op.c == 0.0)
