"""The per-device batch layout (``dips_gb300.dp``) against ``DatasetDict(x, batch_size, num_gpus)``
of the reference (data/data_management.py:79-159), no GPU.

``tests/golden/ref_dataset_layout.npz`` holds the reference's ``batched_data`` for nine
(points, batch size, devices) cases -- uneven splits, a batch larger than a device's run, runs that
end past the last point, a padded extra batch on every device -- written by the reference's
unmodified module on the numpy stand-in for jax, with its padding points replaced by a marker
value (the reference draws them with jax's PRNG; this library draws them with numpy).  Every
device's points, batch size, batch count and padding positions must match exactly.  When the
reference checkout is present the fixture is also regenerated and compared (in a subprocess, so
that the stand-in never enters this process).
"""

import os
import subprocess
import sys

import numpy as np
import pytest

from golden import make_reference_golden as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIXTURE = os.path.join(ROOT, "tests", "golden", "ref_dataset_layout.npz")
REF = os.environ.get("JAX_DIPS_REFERENCE", M.DEFAULT_REFERENCE)


def _fixture():
    return dict(np.load(FIXTURE))


def test_device_layout_matches_the_reference():
    from dips_gb300 import dp

    fx = _fixture()
    cases = fx["cases"]
    pad = np.float32(fx["pad"])
    assert len(cases) == len(M.DATA_CASES)
    for i, (n, bs, g) in enumerate(cases):
        ref = fx[f"batched_{i}"]
        x = np.arange(3 * n, dtype=np.float32).reshape(n, 3) / np.float32(7.0)
        assert ref.shape[0] == g
        for rank in range(g):
            mine, b, nb = dp.device_points(x, int(bs), rank, int(g), lambda c: np.full((c, 3), pad, np.float32))
            assert (nb, b) == ref.shape[1:3], (n, bs, g, rank)
            np.testing.assert_array_equal(mine, ref[rank].reshape(-1, 3), err_msg=f"{(n, bs, g, rank)}")
        # every point is on some device, once
        real = ref.reshape(-1, 3)
        real = real[real[:, 0] != pad]
        assert real.shape[0] == n and np.unique(real[:, 0]).size == n


_REGEN = r"""
import sys, numpy as np
sys.path[:0] = [sys.argv[1] + "/oracle", sys.argv[1] + "/jax-dips_gb300", sys.argv[1] + "/tests"]
from golden import make_reference_golden as M
out = M.run_data_case(sys.argv[2])
ref = np.load(sys.argv[1] + "/tests/golden/ref_dataset_layout.npz")
bad = [k for k in out if not np.array_equal(np.asarray(out[k]), ref[k])]
print("BAD" if bad or set(out) != set(ref.files) else "OK", bad)
"""


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "jax_dips")), reason="the reference checkout is not available")
def test_layout_fixture_regenerates_from_the_reference():
    out = subprocess.run([sys.executable, "-W", "ignore", "-c", _REGEN, ROOT, REF], capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    assert out.stdout.strip().startswith("OK"), out.stdout[-2000:]
