"""The C ABI library builds for sm_103a, loads on a host without a GPU, and exports every
entry point include/dips.h declares (no compute calls here)."""

import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fname in os.listdir(os.path.join(ROOT, "include")):
        if not fname.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fname)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(dips_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("dips_last_error", "dips_phi_trilinear", "dips_geometry_assemble", "dips_residual_fwd",
                     "dips_residual_bwd", "dips_train_step", "dips_adam_step"):
        assert required in names


def test_library_loads_and_exports_all_declared_symbols():
    from dips_gb300 import _lib

    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"symbols declared in include/ but not exported: {missing}"
    assert lib.dips_version().startswith(b"dips_gb300")


def test_arch_table_and_workspace_query():
    from dips_gb300 import _lib
    from dips_gb300.nn import Arch, n_params

    lib = _lib.load()
    for a in (Arch(1, 1, 2, 10), Arch(3, 32, 3, 32), Arch(2, 16, 2, 16), Arch(2, 8, 2, 8), Arch(4, 64, 4, 64)):
        assert lib.dips_arch_supported(a.ctype()) == 1
        assert lib.dips_num_params(a.ctype()) == n_params(a)
    assert lib.dips_arch_supported(Arch(2, 64, 2, 64).ctype()) == 0
    small = lib.dips_step_workspace_bytes(Arch().ctype(), 1000, 7000)
    big = lib.dips_step_workspace_bytes(Arch().ctype(), 1000, 70000)
    assert 0 < small < big


def test_argument_errors_are_reported_without_a_gpu():
    from dips_gb300 import _lib

    lib = _lib.load()
    # null pointers are rejected on the host before any CUDA call
    st = lib.dips_phi_ghost_layer(None, 4, 4, 4, None, None)
    assert st == 1
    assert b"null" in lib.dips_last_error()
    a = _lib.ArchT(5, 5, 5, 5)
    st = lib.dips_mlp_eval(a, _lib.c_void_p(8), _lib.c_void_p(8), _lib.c_void_p(8), 4, _lib.c_void_p(8), None, None)
    assert st == 4 and b"no kernel compiled" in lib.dips_last_error()


def test_noalloc_step_rejects_bad_sizes_on_the_host():
    """dips_train_step_noalloc checks the batch and its built-in scratch limit before any CUDA
    call, so both rejections are visible without a GPU."""
    from dips_gb300 import _lib

    lib = _lib.load()
    a = _lib.ArchT(3, 32, 3, 32)
    p = _lib.c_void_p(8)
    st = lib.dips_train_step_noalloc(a, None, p, p, p, p, None, None, 0, 0, p, None, None)
    assert st == 1 and b"bad batch" in lib.dips_last_error()
    need = lib.dips_step_workspace_bytes(a, 4096, 10**8)
    assert need > 64 << 20
    st = lib.dips_train_step_noalloc(a, None, p, p, p, p, None, None, 4096, 10**8, p, None, None)
    assert st == 3 and b"built-in" in lib.dips_last_error()


# entry points that return a size, a count, a string or a previous setting rather than a status
_NOT_STATUS = {"dips_version", "dips_last_error", "dips_tc_set_wait_limit", "dips_num_params", "dips_arch_supported",
               "dips_step_workspace_bytes", "dips_bicgstab_workspace_bytes", "dips_instances_table_bytes",
               "dips_geometry_assemble_scratch_bytes", "dips_xla_workspace_bytes", "dips_xla_set_status_fn"}


def _status_entry_points():
    from dips_gb300 import _lib

    return [n for n in sorted(_lib._SIGS) if n not in _NOT_STATUS]


@pytest.mark.parametrize("name", _status_entry_points())
def test_null_pointers_are_rejected_on_the_host(name):
    """Every status-returning entry point, called with every pointer NULL and every size 1,
    returns a non-zero status with a message (the XLA handlers, which return nothing, record
    the message), before any CUDA call: no host dereference of a NULL struct pointer and no
    launch on NULL device pointers."""
    import ctypes

    from dips_gb300 import _lib

    lib = _lib.load()
    res, args = _lib._SIGS[name]
    vals = []
    for a in args:
        if a in (ctypes.c_float, ctypes.c_double):
            vals.append(1.0)
        elif a is ctypes.c_void_p or a is ctypes.c_char_p or issubclass(a, (ctypes._Pointer, ctypes._CFuncPtr)):
            vals.append(None)
        else:
            vals.append(1)
    lib.dips_last_error()
    st = getattr(lib, name)(*vals)
    msg = lib.dips_last_error().decode()
    if res is None:  # XLA custom-call handlers
        assert msg.startswith("dips_xla"), msg
        return
    assert st != 0, name
    assert msg and msg != "no error", name


def test_size_queries_without_a_shape_return_zero():
    from dips_gb300 import _lib

    lib = _lib.load()
    assert lib.dips_num_params(None) == -1
    assert lib.dips_arch_supported(None) == 0
    assert lib.dips_step_workspace_bytes(None, 1, 1) == 0
    assert lib.dips_xla_workspace_bytes(None, 1, 1) == 0
