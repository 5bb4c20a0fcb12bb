"""The oracle's level-set interpolants against the reference's own (no GPU).

``tests/golden/ref_interp_nodal16.npz`` holds ``multilinear_interpolation`` (interpolate.py:
906-1021) and ``nonoscillatory_quadratic_interpolation`` (:572-759) of a seeded nodal field on the
16^3 grid, computed by the reference's unmodified module on the numpy stand-in for jax, at points
inside the box, in its first and last cells (where both clamp the cell index and extrapolate),
beyond it, and on nodes.  The oracle's restatements must reproduce every value bit for bit; the
CUDA kernels (``dips_phi_trilinear``, ``dips_phi_quadratic``) are held bit-exact to these same
restatements on the GPU, inside and beyond the box.  When the reference checkout is present the
fixture is also regenerated and compared (in a subprocess, so that the stand-in never enters
this process).
"""

import os
import subprocess
import sys

import numpy as np
import pytest

from golden import make_reference_golden as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
FIXTURE = os.path.join(ROOT, "tests", "golden", "ref_interp_nodal16.npz")
REF = os.environ.get("JAX_DIPS_REFERENCE", M.DEFAULT_REFERENCE)


def test_oracle_interpolants_match_the_reference_bit_for_bit():
    import nbm_oracle as O

    fx = dict(np.load(FIXTURE))
    n = int(fx["n"])
    x = O.linspace_f32(-1.0, 1.0, n)
    T = O.Trilinear(fx["u"], x, x, x)
    pts = fx["pts"]
    np.testing.assert_array_equal(np.asarray(T(pts), np.float32).reshape(-1), fx["trilinear"])
    np.testing.assert_array_equal(np.asarray(T.quadratic(pts), np.float32).reshape(-1), fx["quadratic"])
    # the fixture covers the clamped first and last cells and points beyond the box
    assert (pts < -1.0).any() and (pts > 1.0).any()
    assert ((pts > -1.0) & (pts < -1.0 + 2.0 / (n - 1))).any()


_REGEN = r"""
import sys, numpy as np
sys.path[:0] = [sys.argv[1] + "/oracle", sys.argv[1] + "/jax-dips_gb300", sys.argv[1] + "/tests"]
from golden import make_reference_golden as M
out = M.run_interp_case(sys.argv[2])
ref = np.load(sys.argv[1] + "/tests/golden/ref_interp_nodal16.npz")
bad = [k for k in out if not np.array_equal(np.asarray(out[k]), ref[k])]
print("BAD" if bad or set(out) != set(ref.files) else "OK", bad)
"""


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "jax_dips")), reason="the reference checkout is not available")
def test_interpolant_fixture_regenerates_from_the_reference():
    out = subprocess.run([sys.executable, "-W", "ignore", "-c", _REGEN, ROOT, REF], capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    assert out.stdout.strip().startswith("OK"), out.stdout[-2000:]
