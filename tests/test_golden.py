"""The oracle against its committed golden fixtures (tests/golden/*.npz, written by
tests/golden/make_golden.py): geometry flags, face coefficients, the interface integral, the
seeded parameters, and the loss and gradient in float64 and float32 on three of the GPU
parity cases.  A change to the oracle that moves any of them fails here."""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from golden import make_golden  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) / np.linalg.norm(b))


@pytest.mark.parametrize("key", sorted(make_golden.CASES))
def test_oracle_reproduces_golden_fixture(key):
    gold = np.load(os.path.join(HERE, "golden", key + ".npz"))
    out = make_golden.compute(make_golden.CASES[key])
    np.testing.assert_array_equal(out["crossed"], gold["crossed"])
    np.testing.assert_array_equal(out["xi"], gold["xi"])
    np.testing.assert_array_equal(out["params"], gold["params"])
    scale = float(np.max(np.abs(gold["coeffs"])))
    np.testing.assert_allclose(out["coeffs"], gold["coeffs"], rtol=1e-5, atol=1e-6 * scale)
    np.testing.assert_allclose(out["beta_int"], gold["beta_int"], rtol=1e-5, atol=1e-6 * float(np.max(np.abs(gold["beta_int"]))))
    assert abs(out["loss64"] - gold["loss64"]) <= 1e-10 * abs(gold["loss64"])
    assert _rel_l2(out["grad64"], gold["grad64"]) <= 1e-9
    assert abs(out["loss32"] - gold["loss32"]) <= 1e-6 * abs(gold["loss32"])
    assert _rel_l2(out["grad32"], gold["grad32"]) <= 1e-5
    # the fixture's float32 loss and gradient are within the parity bars of its float64 ones
    assert abs(float(gold["loss32"]) - float(gold["loss64"])) <= 1e-5 * abs(float(gold["loss64"]))
    assert _rel_l2(gold["grad32"], gold["grad64"]) <= 1e-4


def test_golden_fixture_catches_a_planted_flux_jump_sign(monkeypatch):
    """A mistake planted in the oracle: the flux jump beta with the opposite sign convention
    (mu+ dn u+ - mu- dn u- instead of the reference problems' -(mu+ dn u+ - mu- dn u-)).  The
    geometry does not depend on beta and still matches; the interface integral, the loss and
    the gradient move beyond the parity bars (loss 1e-5, gradient 1e-4 relative)."""
    import _parity

    make_problem = _parity.make_problem

    def flipped(name):
        fns = dict(make_problem(name))
        beta = fns["beta"]
        fns["beta"] = lambda r: -beta(r)
        return fns

    monkeypatch.setattr(_parity, "make_problem", flipped)
    key = "sphere16_1x1_2x10_l0"
    gold = np.load(os.path.join(HERE, "golden", key + ".npz"))
    out = make_golden.compute(make_golden.CASES[key])
    np.testing.assert_array_equal(out["crossed"], gold["crossed"])
    np.testing.assert_allclose(out["coeffs"], gold["coeffs"], rtol=1e-5, atol=1e-6 * float(np.max(np.abs(gold["coeffs"]))))
    np.testing.assert_allclose(out["beta_int"], -gold["beta_int"], rtol=1e-6)
    # measured: 7.1e-4 (loss) and 2.5e-3 (gradient), both beyond the parity bars (1e-5, 1e-4)
    assert abs(out["loss64"] - gold["loss64"]) > 10 * 1e-5 * abs(gold["loss64"])
    assert _rel_l2(out["grad64"], gold["grad64"]) > 10 * 1e-4
