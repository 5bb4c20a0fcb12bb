"""Writes the golden fixtures of this directory: the oracle's outputs on three of the GPU
parity cases (tests/test_gpu_parity.py), so that any later change to the oracle that moves
its results is caught (tests/test_golden.py).

The reference itself (jax 0.4.13, dm-haiku, optax) cannot be imported here, so these are
outputs of the oracle, not of the reference: they pin the oracle against drift.  The
oracle's own pins are the reference's known-answer test for the geometry
(tests/test_geometric_integrations.py:172-182 of the reference), numpy's pinv and
central differences (tests/test_oracle.py).

Per case (one .npz each):
  crossed   int8  [N]       cell-crossing flag of every grid point (geom_pp.py:203-263)
  xi        int32 [M]       indices of the crossed points
  coeffs    f32   [M, 26]   face coefficients and volumes at the crossed points (geom_pp.py:464-1009)
  beta_int  f32   [M]       interface integral of beta at the crossed points (geom_pp.py:383-461)
  params    f32   [P]       the parameter vector (seeded init)
  loss64, grad64            loss and gradient in float64 (trainer.py:892-912, :783-789)
  loss32, grad32            the same in float32

Run:  python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import _parity  # noqa: E402

CASES = {
    "sphere16_1x1_2x10_l0": dict(name="sphere", n=16, arch=(1, 1, 2, 10), level=0),
    "star20_2x16_l1": dict(name="star", n=20, arch=(2, 16, 2, 16), level=1),
    "sphere20_3x32_l0": dict(name="sphere", n=20, arch=(3, 32, 3, 32), level=0),
}


def compute(spec):
    import torch

    case = _parity.build_case(spec["name"], n=spec["n"], arch=spec["arch"], level=spec["level"])
    rg = case.oracle_geometry()
    crossed = np.asarray(rg.crossed_p, np.int8)
    xi = np.nonzero(crossed == 0)[0].astype(np.int32)
    l64, g64 = case.oracle_loss_grad(torch.float64)
    l32, g32 = case.oracle_loss_grad(torch.float32)
    return dict(
        crossed=crossed,
        xi=xi,
        coeffs=np.asarray(rg.coeffs, np.float32)[xi],
        beta_int=np.asarray(rg.beta_int, np.float32)[xi],
        params=np.asarray(case.params, np.float32),
        loss64=np.float64(l64),
        grad64=np.asarray(g64, np.float64),
        loss32=np.float32(l32),
        grad32=np.asarray(g32, np.float32),
    )


def main():
    for key, spec in CASES.items():
        out = compute(spec)
        path = os.path.join(HERE, key + ".npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {os.path.getsize(path)} bytes, {out['xi'].size} crossed points, loss {out['loss64']:.9e}")


if __name__ == "__main__":
    main()
