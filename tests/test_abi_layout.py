"""The Python (ctypes) mirrors of the C ABI's structs have the header's layout: size and the
offset of every field, measured by a small C program compiled here against include/dips.h
(no GPU).  A mismatch would pass wrong pointers across the boundary without any error."""

import ctypes
import os
import shutil
import subprocess

import pytest

from dips_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MIRRORS = {
    "dips_levelset_t": _lib.LevelSetT,
    "dips_coeffs_t": _lib.CoeffsT,
    "dips_records_t": _lib.RecordsT,
    "dips_arch_t": _lib.ArchT,
    "dips_adam_t": _lib.AdamT,
    "dips_instance_t": _lib.InstanceT,
    "dips_krylov_stats_t": _lib.KrylovStatsT,
    "dips_xla_desc_t": _lib.XlaDescT,
}


def _cuda_include():
    for d in ("/usr/local/cuda/include", os.path.join(os.environ.get("CUDA_HOME", ""), "include")):
        if d and os.path.exists(os.path.join(d, "cuda_runtime.h")):
            return d
    return None


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    inc = _cuda_include()
    if not cc or not inc:
        pytest.skip("needs a C compiler and the CUDA headers")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dips.h"', "int main(void) {"]
    for cname, mirror in MIRRORS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in mirror._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), "-I", inc, str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, what, value = line.split()
        got[(cname, what)] = int(value)
    return got


@pytest.mark.parametrize("cname", sorted(MIRRORS))
def test_ctypes_mirror_matches_the_header(c_layout, cname):
    mirror = MIRRORS[cname]
    assert ctypes.sizeof(mirror) == c_layout[(cname, "size")], cname
    for fname, _ in mirror._fields_:
        assert getattr(mirror, fname).offset == c_layout[(cname, fname)], (cname, fname)
