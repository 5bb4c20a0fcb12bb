"""Nonlinear operators N-(u-) V- + N+(u+) V+ (discretization.py:369) on the GPU, against the oracle.

The reference-generated fixture ``ref_sphere16_sinh_3x32_l0`` (the sphere with N-(u) = 300 sinh(u)
and N+(u) = 100 sinh(u), output biases shifted so that u is of order one) is checked by
``test_gpu_reference.py`` like every other fixture.  Here the same operators run through the other
engines (2x16 tile engine, 4x64 TF32 engine, a per-job shape) against the FP64 oracle, at both
stencil levels, and the entry points that cannot take them refuse the records instead of ignoring
the term.  With nonlinear operators every point takes the general path (expansion, per-job
forward, general residual and adjoint); the term and its derivative are formed in the general
residual kernel.

Bars: the loss to 1e-5 relative and the gradient to 1e-4 of its norm on the FP32 engines.  On
the TF32 engine u is of order one here and carries TF32's relative error (10 mantissa bits
through four layers), which the large operator (300 sinh u) amplifies: 1e-3 and 1e-2.  Leaving
the term out moves the gradient by 0.3-6 % of its norm.
"""

import ctypes

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _sinh_case(arch, level=0):
    from golden import make_reference_golden as M

    import nbm_loss as L

    case = _parity.Case("sphere_sinh", 16, arch, level=level, fns=M.problem("sphere_sinh"))
    # output biases moved as in the fixture, so that u is of order one
    a = case.arch
    n_m = sum(i * o + o for i, o in L.net_sizes(*a.net("m")))
    n_p = sum(i * o + o for i, o in L.net_sizes(*a.net("p")))
    p = case.params.copy()
    p[n_m - 1] += np.float32(0.8)
    p[n_m + n_p - 1] -= np.float32(0.6)
    case.params = p
    return case


@pytest.mark.parametrize("arch,level", [((2, 16, 2, 16), 0), ((3, 32, 3, 32), 1), ((4, 64, 4, 64), 0),
                                        ((1, 1, 2, 10), 0)])
def test_nonlinear_loss_and_gradient_match_the_oracle(arch, level):
    case = _sinh_case(arch, level)
    tf32 = arch == (4, 64, 4, 64)
    lo, go = case.oracle_loss_grad(torch.float64)
    lg, gg = case.gpu_loss_grad()
    assert abs(lg - lo) <= (1e-3 if tf32 else 1e-5) * abs(lo), (lg, lo)
    gn = float(np.linalg.norm(go))
    assert float(np.max(np.abs(np.asarray(gg, np.float64) - go))) <= (1e-2 if tf32 else 1e-4) * gn
    # the term matters: without it the oracle's gradient moves by 3-6 % of its norm at h = dx and
    # 0.3 % at h = dx/2, where the cell volumes are 8 times smaller (twenty times the FP32 bar)
    base = _parity.Case("sphere", 16, arch, level=level, fns={k: v for k, v in case.fns.items()
                                                               if k not in ("nl_m", "nl_p")}, params=case.params)
    _, gb = base.oracle_loss_grad(torch.float64)
    assert float(np.linalg.norm(np.asarray(gb) - go)) > 2e-3 * gn


def test_nonlinear_records_refuse_the_linear_only_entry_points():
    from dips_gb300 import _lib, krylov, ops

    case = _sinh_case((3, 32, 3, 32))
    lvl = case.gpu_level()
    assert lvl.desc.nl_pt and lvl.desc.nl_w and list(lvl.desc.nl_kind) == [1, 1]
    assert list(lvl.desc.nl_c) == [300.0, 100.0]
    # the plain method needs a linear operator
    with pytest.raises(_lib.DipsError, match="not linear"):
        krylov.bicgstab(lvl, (16, 16, 16), max_iter=5)
    # the coefficient derivative does not differentiate the nonlinear term
    tan = lvl.coefficient_tangent({"mu_p": lambda r: 1.0})
    params = torch.as_tensor(case.params, device="cuda")
    with pytest.raises(_lib.DipsError, match="nonlinear"):
        ops.loss_coefficient_derivative(case.gpu_arch(), params, lvl, tan)
    torch.cuda.synchronize()
    # the library is still usable
    lg, _ = case.gpu_loss_grad()
    assert np.isfinite(lg)


def test_batched_instance_step_refuses_nonlinear_records():
    from dips_gb300 import _lib, ops

    case = _sinh_case((2, 16, 2, 16))
    lvl = case.gpu_level()
    arch = case.gpu_arch()
    params = torch.as_tensor(case.params, device="cuda")
    B = 256
    opt = ops.AdamState(params.numel(), lr=1e-3)
    ws = ops.StepWorkspace(arch, B, lvl.max_jobs(B), torch.device("cuda"))
    ids = torch.arange(B, dtype=torch.int32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    arr = (_lib.InstanceT * 1)()
    arr[0] = _lib.InstanceT(ctypes.addressof(lvl.desc), _lib.ptr(ids), B, 0, 0, -1, _lib.ptr(params),
                            _lib.ptr(opt.mu), _lib.ptr(opt.nu), _lib.ptr(opt.count), _lib.ptr(ws.buf), ws.nbytes,
                            _lib.ptr(loss), None)
    lib = _lib.load()
    nbytes = int(lib.dips_instances_table_bytes(1))
    table = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    st = lib.dips_instances_prepare(arch.ctype(), arr, 1, _lib.ptr(table), nbytes, _lib.stream_handle())
    assert st != 0
    assert "nonlinear" in lib.dips_last_error().decode()
