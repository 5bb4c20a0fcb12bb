"""Build and load ``libdips_gb300.so`` (the C ABI declared in include/dips.h).

The library is compiled in-tree with nvcc for sm_103a.  There is no fallback: if
the library cannot be built or loaded, every entry point raises.
"""

from __future__ import annotations

import ctypes
import hashlib
import platform
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)  # jax-dips_gb300/
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libdips_gb300.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
# per translation unit extra flags: the geometry kernels must round every float32
# operation separately (no FMA contraction) to take the reference's discrete decisions
UNITS = {
    "capi.cu": [],
    "geometry.cu": ["-fmad=false"],
    "residual.cu": [],
    "residual_a1_1_2_10.cu": [],
    "residual_a2_8_2_8.cu": [],
    "residual_a2_16_2_16.cu": [],
    "residual_a3_32_3_32.cu": [],
    "krylov.cu": [],
    "residual_static.cu": [],
    "residual_tc.cu": [],
    "precond.cu": [],
    "xla_shim.cu": [],
}

_lock = threading.Lock()
_lib = None


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the dips_gb300 CUDA library cannot be built")


def _sources():
    return [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]


def _fingerprint():
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)) + ["dips.h"]:
        path = os.path.join(CSRC, name) if name != "dips.h" else os.path.join(INCLUDE, "dips.h")
        if os.path.isfile(path):
            h.update(name.encode())
            with open(path, "rb") as f:
                h.update(f.read())
    # the host machine too: a library built on another architecture is never reused
    h.update(repr((ARCH_FLAGS, COMMON_FLAGS, UNITS, platform.machine())).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link the shared library."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    stamp = os.path.join(BUILD_DIR, "stamp.txt")
    fp = _fingerprint()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == fp:
                return LIB_PATH
    nvcc = _nvcc()

    def compile_unit(unit):
        obj = os.path.join(BUILD_DIR, unit.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH_FLAGS, *COMMON_FLAGS, *UNITS[unit], "-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr[-6000:]}")
        return obj, r.stderr

    units = _sources()
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(compile_unit, units))
    objs = [o for o, _ in results]
    tmp = LIB_PATH + ".tmp"
    r = subprocess.run([nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(fp)
    if verbose:
        for _, log in results:
            print(log)
    return LIB_PATH


# ----------------------------------------------------------------------------------------
# ctypes mirror of include/dips.h
# ----------------------------------------------------------------------------------------
c_void_p = ctypes.c_void_p
c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_f32 = ctypes.c_float


class LevelSetT(ctypes.Structure):
    _fields_ = [
        ("phi_gh", c_void_p),
        ("xg", c_void_p),
        ("yg", c_void_p),
        ("zg", c_void_p),
        ("nx", c_i32),
        ("ny", c_i32),
        ("nz", c_i32),
        ("xmin", c_f32),
        ("xmax", c_f32),
        ("ymin", c_f32),
        ("ymax", c_f32),
        ("zmin", c_f32),
        ("zmax", c_f32),
    ]


class CoeffsT(ctypes.Structure):
    _fields_ = [
        (n, c_void_p)
        for n in (
            "mu_m_face",
            "mu_p_face",
            "k_m",
            "k_p",
            "f_m",
            "f_p",
            "g",
            "beta_tri",
            "mu_m_s",
            "mu_p_s",
            "alpha_r",
            "beta_r",
            "mu_m_r",
            "mu_p_r",
        )
    ] + [("beta_origin", c_f32)]


class RecordsT(ctypes.Structure):
    _fields_ = [
        ("pts", c_void_p),
        ("n_pts", c_i64),
        ("h", c_f32 * 3),
        ("lhs0", c_void_p),
        ("diag", c_void_p),
        ("rod", c_void_p),
        ("cnt", c_void_p),
        ("cnt_m", c_void_p),
        ("job_off", c_void_p),
        ("job_code", c_void_p),
        ("job_A", c_void_p),
        ("coeff26", c_void_p),
        ("bulk_rec", c_void_p),
        ("nl_pt", c_void_p),
        ("nl_w", c_void_p),
        ("nl_kind", c_i32 * 2),
        ("nl_c", c_f32 * 2),
    ]


class ArchT(ctypes.Structure):
    _fields_ = [("m_layers", c_i32), ("m_width", c_i32), ("p_layers", c_i32), ("p_width", c_i32),
                ("pre_layers", c_i32), ("pre_width", c_i32), ("pre_scaling", c_f32)]


class AdamT(ctypes.Structure):
    _fields_ = [(n, c_f32) for n in ("lr", "decay_rate", "transition_steps", "max_norm", "b1", "b2", "eps")] + [
        ("kind", c_i32), ("schedule", c_i32)]


OPT_ADAM, OPT_RMSPROP = 0, 1
SCHED_EXPONENTIAL, SCHED_POLYNOMIAL = 0, 1


class InstanceT(ctypes.Structure):
    _fields_ = [
        ("rec", ctypes.c_void_p),
        ("batch_ids", c_void_p),
        ("batch", c_i64),
        ("n_batches", c_i64),
        ("seed", ctypes.c_uint64),
        ("ids_mode", c_i32),
        ("params", c_void_p),
        ("mu", c_void_p),
        ("nu", c_void_p),
        ("count", c_void_p),
        ("workspace", c_void_p),
        ("ws_bytes", ctypes.c_size_t),
        ("loss_out", c_void_p),
        ("grad_out", c_void_p),
    ]


class KrylovStatsT(ctypes.Structure):
    _fields_ = [("iterations", c_i32), ("target_iteration", c_i32), ("breakdown", c_i32),
                ("rel_residual", ctypes.c_double), ("rel_linf", c_f32)]


class XlaDescT(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_uint32), ("version", ctypes.c_uint32), ("arch", ArchT), ("rec", c_void_p),
                ("batch", c_i64), ("max_jobs", c_i64), ("ws_bytes", ctypes.c_uint64)]


# void (*)(XlaCustomCallStatus*, const char*, size_t)
XlaStatusFn = ctypes.CFUNCTYPE(None, c_void_p, ctypes.c_char_p, ctypes.c_size_t)

P = ctypes.POINTER
_SIGS = {
    "dips_last_error": (ctypes.c_char_p, []),
    "dips_version": (ctypes.c_char_p, []),
    "dips_fp32_fma_probe": (c_i32, [c_void_p, c_i32, c_i32, c_void_p]),
    "dips_phi_ghost_layer": (c_i32, [c_void_p, c_i32, c_i32, c_i32, c_void_p, c_void_p]),
    "dips_phi_trilinear": (c_i32, [P(LevelSetT), c_void_p, c_i64, c_void_p, c_void_p]),
    "dips_phi_quadratic": (c_i32, [P(LevelSetT), c_void_p, c_i64, c_void_p, c_void_p]),
    "dips_geometry_classify": (
        c_i32,
        [P(LevelSetT), c_void_p, c_i64, P(c_f32), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    ),
    "dips_geometry_queries": (
        c_i32,
        [P(LevelSetT), c_void_p, c_i64, P(c_f32), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
         c_void_p],
    ),
    "dips_geometry_queries_ex": (
        c_i32,
        [P(LevelSetT), c_void_p, c_i64, P(c_f32), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
         c_void_p, ctypes.c_size_t, c_void_p],
    ),
    "dips_geometry_assemble": (
        c_i32,
        [P(LevelSetT), c_void_p, c_i64, P(c_f32), c_void_p, c_void_p, c_void_p, c_void_p, P(CoeffsT)]
        + [c_void_p] * 9
        + [c_void_p],
    ),
    "dips_geometry_assemble_scratch_bytes": (ctypes.c_size_t, [c_i64]),
    "dips_geometry_assemble_ex": (
        c_i32,
        [P(LevelSetT), c_void_p, c_i64, P(c_f32), c_void_p, c_void_p, c_void_p, c_void_p, P(CoeffsT)]
        + [c_void_p] * 12
        + [ctypes.c_size_t, c_void_p],
    ),
    "dips_geometry_assemble_tangent": (
        c_i32,
        [P(LevelSetT), c_void_p, c_i64, P(c_f32), c_void_p, c_void_p, c_void_p, c_void_p, P(CoeffsT), P(CoeffsT)]
        + [c_void_p] * 4
        + [c_void_p],
    ),
    "dips_loss_coeff_tangent": (
        c_i32,
        [P(ArchT), c_void_p, P(RecordsT), P(RecordsT), c_void_p, c_i64, c_void_p, ctypes.c_size_t, c_void_p,
         c_void_p],
    ),
    "dips_pack_bulk_records": (c_i32, [P(RecordsT), c_void_p, c_void_p]),
    "dips_instances_table_bytes": (ctypes.c_size_t, [c_i32]),
    "dips_instances_prepare": (c_i32, [P(ArchT), P(InstanceT), c_i32, c_void_p, ctypes.c_size_t, c_void_p]),
    "dips_train_step_instances": (c_i32, [P(ArchT), P(AdamT), c_void_p, c_i32, c_i64, c_void_p]),
    "dips_num_params": (c_i32, [P(ArchT)]),
    "dips_arch_supported": (c_i32, [P(ArchT)]),
    "dips_step_workspace_bytes": (ctypes.c_size_t, [P(ArchT), c_i64, c_i64]),
    "dips_residual_fwd": (
        c_i32,
        [P(ArchT), c_void_p, P(RecordsT), c_void_p, c_i64, c_void_p, ctypes.c_size_t, c_void_p, c_void_p, c_void_p],
    ),
    "dips_residual_bwd": (
        c_i32,
        [P(ArchT), c_void_p, P(RecordsT), c_void_p, c_i64, c_void_p, ctypes.c_size_t, c_void_p, c_void_p],
    ),
    "dips_adam_step": (c_i32, [P(ArchT), P(AdamT), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "dips_train_step": (
        c_i32,
        [P(ArchT), P(AdamT), c_void_p, c_void_p, c_void_p, c_void_p, P(RecordsT), c_void_p, c_i64, c_void_p,
         ctypes.c_size_t, c_void_p, c_void_p, c_void_p],
    ),
    "dips_train_step_profiled": (
        c_i32,
        [P(ArchT), P(AdamT), c_void_p, c_void_p, c_void_p, c_void_p, P(RecordsT), c_void_p, c_i64, c_void_p,
         ctypes.c_size_t, c_void_p, c_void_p, c_void_p, c_i32, c_void_p],
    ),
    "dips_train_step_noalloc": (
        c_i32,
        [P(ArchT), P(AdamT), c_void_p, c_void_p, c_void_p, c_void_p, P(RecordsT), c_void_p, c_i64, c_i64, c_void_p,
         c_void_p, c_void_p],
    ),
    "dips_autotune": (
        c_i32,
        [P(ArchT), c_void_p, P(RecordsT), c_void_p, c_i64, c_void_p, ctypes.c_size_t, P(c_i32), c_void_p],
    ),
    "dips_batch_ids": (c_i32, [c_i64, c_i64, ctypes.c_uint64, c_i64, c_i64, c_void_p, c_void_p]),
    "dips_batch_ids_device": (c_i32, [c_i64, c_i64, c_i64, ctypes.c_uint64, c_i32, c_void_p, c_void_p, c_void_p]),
    "dips_mlp_eval": (c_i32, [P(ArchT), c_void_p, c_void_p, c_void_p, c_i64, c_void_p, c_void_p, c_void_p]),
    "dips_fv_residual": (c_i32, [P(RecordsT), c_i32, c_i32, c_i32, c_void_p, c_i32, c_void_p, c_void_p]),
    "dips_bicgstab": (
        c_i32,
        [P(RecordsT), c_i32, c_i32, c_i32, c_void_p, c_void_p, c_i32, ctypes.c_double, c_i32, c_f32, c_void_p,
         ctypes.c_size_t, P(KrylovStatsT), c_void_p],
    ),
    "dips_bicgstab_workspace_bytes": (ctypes.c_size_t, [c_i64]),
    "dips_tc_set_wait_limit": (ctypes.c_uint32, [ctypes.c_uint32]),
    "dips_xla_workspace_bytes": (ctypes.c_size_t, [P(ArchT), c_i64, c_i64]),
    "dips_xla_make_desc": (c_i32, [P(ArchT), P(RecordsT), c_i64, c_i64, P(XlaDescT)]),
    "dips_xla_set_status_fn": (None, [XlaStatusFn]),
    "dips_xla_loss_fwd": (None, [c_void_p, P(c_void_p), c_void_p, ctypes.c_size_t, c_void_p]),
    "dips_xla_loss_bwd": (None, [c_void_p, P(c_void_p), c_void_p, ctypes.c_size_t, c_void_p]),
}


def exported_symbols():
    """Names of the C ABI entry points (as declared in include/dips.h)."""
    return sorted(_SIGS)


def load(build_if_needed: bool = True):
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = build() if build_if_needed else LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError(f"dips_gb300 CUDA library missing at {path}; call build() first")
        lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class DipsError(RuntimeError):
    pass


def check(status: int, what: str):
    if status != 0:
        msg = load().dips_last_error().decode(errors="replace")
        raise DipsError(f"{what} failed (status {status}): {msg}")


def stream_handle(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())
