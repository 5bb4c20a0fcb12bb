"""VTK structured-grid output of solution fields (utils/io.py:62-88): files written for a grid
read back to the same coordinates and values, in VTK's point order (x fastest)."""

import numpy as np

from dips_gb300 import io, mesh


def test_vtk_manual_round_trip(tmp_path):
    g = mesh.uniform_grid(4)
    X, Y, Z = np.meshgrid(g.x, g.y, g.z, indexing="ij")
    sol = (X + 10 * Y + 100 * Z).astype(np.float32)
    grad = np.stack([X, Y, Z], -1).astype(np.float32)
    fname = io.write_vtk_manual(g, {"sol": sol, "grad": grad, "flat": sol.reshape(-1)}, str(tmp_path / "dump"))
    back = io.read_vts(fname)
    # VTK order: x fastest, then y, then z
    ref_pts = np.stack([X, Y, Z], -1).transpose(2, 1, 0, 3).reshape(-1, 3)
    np.testing.assert_array_equal(back["Points"], ref_pts)
    np.testing.assert_array_equal(back["sol"], sol.transpose(2, 1, 0).reshape(-1))
    np.testing.assert_array_equal(back["flat"], sol.transpose(2, 1, 0).reshape(-1))
    np.testing.assert_array_equal(back["grad"], grad.transpose(2, 1, 0, 3).reshape(-1, 3))
    head = open(fname, "rb").read(400).decode(errors="ignore")
    assert 'type="StructuredGrid"' in head and 'WholeExtent="0 3 0 3 0 3"' in head


def test_vtk_solution_series(tmp_path):
    g = mesh.uniform_grid(3)
    log = {"U": [np.arange(27, dtype=np.float32) * k for k in range(3)]}
    files = io.write_vtk_solution(g, log, str(tmp_path), maxsteps=2)
    assert [f.split("/")[-1] for f in files] == ["solution0000.vts", "solution0001.vts"]
    np.testing.assert_array_equal(io.read_vts(files[1])["sol"],
                                  (np.arange(27, dtype=np.float32)).reshape(3, 3, 3).transpose(2, 1, 0).reshape(-1))
