"""The two-pass assembly (bulk points first, then the listed points next to the interface) writes
the same records as the one-pass assembly, bit for bit: every point runs the same code in either
case, only the thread that runs it differs.  Checked on the sphere at both stencil levels and on
the star, with and without the nonlinear operators' outputs."""

import numpy as np
import pytest

import _parity

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,level,nl", [("sphere", 0, False), ("sphere", 1, False), ("star", 0, False),
                                           ("sphere_sinh", 0, True)])
def test_two_pass_assembly_matches_one_pass(name, level, nl):
    from golden import make_reference_golden as M

    from dips_gb300 import _lib

    fns = M.problem(name) if nl else _parity.make_problem(name)
    case = _parity.Case(name, 24, (1, 1, 2, 10), level=level, fns=fns)
    lvl = case.gpu_level()  # assembled in two passes (scratch given)
    lib = _lib.load()
    P = _lib.ptr
    tri_off, xs_off, _, _, _, co, _ = lvl._geo
    n = lvl.n
    f32 = dict(dtype=torch.float32, device="cuda")
    out = dict(lhs0=torch.empty(n, **f32), diag=torch.empty(n, **f32), rod=torch.empty(n, **f32),
               cnt=torch.empty(n, dtype=torch.int32, device="cuda"),
               cnt_m=torch.empty(n, dtype=torch.int32, device="cuda"),
               job_code=torch.zeros_like(lvl.job_code), job_A=torch.zeros_like(lvl.job_A),
               coeff26=torch.empty_like(lvl.coeff26), beta_int=torch.empty_like(lvl.beta_int))
    nl_pt = torch.empty_like(lvl.nl_pt) if nl else None
    nl_w = torch.zeros_like(lvl.nl_w) if nl else None
    st = lib.dips_geometry_assemble_ex(lvl.ls.desc, P(lvl.pts), n, lvl._hc(), P(lvl.flags), P(tri_off), P(xs_off),
                                       P(lvl.job_off), co, P(out["lhs0"]), P(out["diag"]), P(out["rod"]),
                                       P(out["cnt"]), P(out["cnt_m"]), P(out["job_code"]), P(out["job_A"]),
                                       P(out["coeff26"]), P(out["beta_int"]), P(nl_pt), P(nl_w), None, 0,
                                       _lib.stream_handle())
    assert st == 0, lib.dips_last_error()
    torch.cuda.synchronize()
    # the job slots that were written (a point's capacity may exceed its jobs; unused slots of
    # job_code are left as allocated)
    off = lvl.job_off.cpu().numpy()
    cnt, cm = out["cnt"].cpu().numpy(), out["cnt_m"].cpu().numpy()
    used = np.zeros(lvl.job_code.numel(), bool)
    for i in range(n):
        used[off[i]:off[i] + cm[i]] = True
        used[off[i + 1] - (cnt[i] - cm[i]):off[i + 1]] = True
    for k, v in out.items():
        a = getattr(lvl, k).cpu().numpy()
        b = v.cpu().numpy()
        if k == "job_code":
            a, b = a[used], b[used]
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8), err_msg=k)
    if nl:
        np.testing.assert_array_equal(lvl.nl_pt.cpu().numpy(), nl_pt.cpu().numpy())
        np.testing.assert_array_equal(lvl.nl_w.cpu().numpy(), nl_w.cpu().numpy())
    # the heavy points were a small part of the grid and both passes had work
    f = lvl.flags.cpu().numpy().astype(np.uint32)
    heavy = np.zeros(n, bool)
    for j in range(7):
        heavy |= ((f >> (4 + 2 * j)) & 3) == 1
    assert 0 < heavy.sum() < n // 2


@pytest.mark.parametrize("name,level", [("sphere", 0), ("star", 1)])
def test_listed_queries_match_one_pass(name, level):
    from dips_gb300 import _lib

    case = _parity.Case(name, 24, (1, 1, 2, 10), level=level, fns=_parity.make_problem(name))
    lvl = case.gpu_level()  # queries of the listed points (scratch given)
    lib = _lib.load()
    P = _lib.ptr
    tri_off, xs_off, tri_pts, xs_pts, xr_pts, _, _ = lvl._geo
    a = [torch.full((max(t.shape[0], 1), 3), float("nan"), dtype=torch.float32, device="cuda")
         for t in (tri_pts, xs_pts, xr_pts)]
    st = lib.dips_geometry_queries(lvl.ls.desc, P(lvl.pts), lvl.n, lvl._hc(), P(lvl.flags), P(tri_off), P(xs_off),
                                   P(a[0]), P(a[1]), P(a[2]), _lib.stream_handle())
    assert st == 0, lib.dips_last_error()
    torch.cuda.synchronize()
    for got, ref in zip((tri_pts, xs_pts, xr_pts), a):
        k = got.shape[0]
        assert k > 0
        np.testing.assert_array_equal(got.cpu().numpy().view(np.uint32), ref[:k].cpu().numpy().view(np.uint32))
