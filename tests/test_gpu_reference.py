"""CUDA path vs golden vectors computed by the reference's own code, through the C ABI.

The fixtures ``tests/golden/ref_*.npz`` hold outputs of the reference's unmodified
discretization and geometry modules (``tests/golden/make_reference_golden.py``) for a seeded batch
of grid points: cell values, interface integrals, crossing flags, per-point [lhs/diag, rhs/diag],
the loss with x64 off and on, and three directional derivatives of the x64 loss.  The CUDA path
gets the same phi samples, parameters and batch.  Cases cover the configuration-1 and -2 sphere,
the configuration-3 star (variable mu, k+ = 1), the reference's own sphere and star problems and
a sphere with constant mu- = 10 > mu+ = 1 (all three take the mu- > mu+ extrapolation branch of
discretization.py:464-486), the configuration-5 blob on the 4x64 TF32 engine and an LPBE molecule
on the 2x16 engine.

Bars: crossing flags exact; cell values and interface integrals to 1e-5 relative (coefficient
callables evaluated by torch on the GPU against numpy on the host); residuals to 3e-5 of their
scale; the loss to 1e-5 relative; each directional derivative to 1e-4 of the gradient norm
(FP32 engines) or 1e-3 (the TF32 engine, whose operands carry 10 mantissa bits).
"""

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KEYS = _parity.reference_fixtures()


@pytest.mark.parametrize("key", KEYS)
def test_cuda_path_matches_reference_fixture(key):
    case, fx = _parity.reference_case(key)
    tf32 = tuple(int(v) for v in fx["arch"]) == (4, 64, 4, 64)
    ids = fx["ids"].astype(np.int64)
    lvl = case.gpu_level()

    f = lvl.flags.cpu().numpy().astype(np.uint32)[ids]
    cp = ((f >> 1) & 3).astype(np.int64) - 1
    np.testing.assert_array_equal(cp, fx["crossed"].astype(np.int64))

    c26 = lvl.coeff26.cpu().numpy()[ids]
    scale = float(np.max(np.abs(fx["coeff26"])))
    np.testing.assert_allclose(c26, fx["coeff26"], rtol=1e-5, atol=1e-6 * scale)
    b = lvl.beta_int.cpu().numpy()[ids]
    fin = np.isfinite(fx["beta_int"])
    np.testing.assert_array_equal(np.isfinite(b), fin)
    if fin.any():
        bs = float(np.max(np.abs(fx["beta_int"][fin])))
        np.testing.assert_allclose(b[fin], fx["beta_int"][fin], rtol=1e-5, atol=1e-6 * bs)

    res = case.gpu_residual()
    ref = fx["lhs_rhs"][:, 0] - fx["lhs_rhs"][:, 1]
    rs = float(np.max(np.abs(ref)))
    err = float(np.max(np.abs(res - ref)))
    assert err <= (1e-4 if tf32 else 3e-5) * rs, (err, rs)

    lg, gg = case.gpu_loss_grad()
    assert abs(lg - float(fx["loss32"])) <= 1e-5 * abs(float(fx["loss32"])), (lg, float(fx["loss32"]))
    gg = np.asarray(gg, np.float64)
    d = fx["dirs"].astype(np.float64) @ gg
    tol = (1e-3 if tf32 else 1e-4) * float(np.linalg.norm(gg))
    np.testing.assert_allclose(d, fx["dloss64"], rtol=0, atol=tol)
