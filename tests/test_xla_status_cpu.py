"""The XLA custom-call handlers report a malformed call through XlaCustomCallStatusSetFailure
found in the process's global symbol scope, as jaxlib provides it (no GPU: the handler rejects the
descriptor before any CUDA call).

A stub library compiled here exports ``XlaCustomCallStatusSetFailure`` (it records the message and
the status pointer) and is loaded with global scope in a fresh process before ``libdips_gb300``;
the handler, given an ``opaque`` of the wrong size and then a descriptor with the wrong magic,
must hand both failures to the stub with the status pointer it was given."""

import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STUB = r"""
#include <stddef.h>
#include <string.h>
static char g_msg[1024];
static void* g_status;
static int g_calls;
void XlaCustomCallStatusSetFailure(void* status, const char* message, size_t len) {
  if (len >= sizeof(g_msg)) len = sizeof(g_msg) - 1;
  memcpy(g_msg, message, len);
  g_msg[len] = 0;
  g_status = status;
  ++g_calls;
}
const char* stub_message(void) { return g_msg; }
void* stub_status(void) { return g_status; }
int stub_calls(void) { return g_calls; }
"""

SCRIPT = r"""
import ctypes, sys
stub = ctypes.CDLL(sys.argv[1], mode=ctypes.RTLD_GLOBAL)
stub.stub_message.restype = ctypes.c_char_p
stub.stub_status.restype = ctypes.c_void_p
sys.path.insert(0, sys.argv[2])
from dips_gb300 import _lib
lib = _lib.load(build_if_needed=False)
status = ctypes.create_string_buffer(16)
bufs = (ctypes.c_void_p * 5)()
lib.dips_xla_loss_fwd(None, bufs, ctypes.cast(ctypes.create_string_buffer(8), ctypes.c_void_p), 8,
                      ctypes.cast(status, ctypes.c_void_p))
print(stub.stub_calls(), stub.stub_status() == ctypes.addressof(status), stub.stub_message().decode())
d = _lib.XlaDescT()
d.magic = 0x12345678
d.version = 1
lib.dips_xla_loss_bwd(None, bufs, ctypes.cast(ctypes.byref(d), ctypes.c_void_p), ctypes.sizeof(d),
                      ctypes.cast(status, ctypes.c_void_p))
print(stub.stub_calls(), stub.stub_status() == ctypes.addressof(status), stub.stub_message().decode())
"""


def test_handler_failure_goes_to_the_global_status_setter(tmp_path):
    from dips_gb300 import _lib

    _lib.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("needs a C compiler")
    src = tmp_path / "stub.c"
    so = tmp_path / "libxlastub.so"
    src.write_text(STUB)
    subprocess.run([cc, "-shared", "-fPIC", "-o", str(so), str(src)], check=True, capture_output=True)
    out = subprocess.run([sys.executable, "-c", SCRIPT, str(so), os.path.join(ROOT, "jax-dips_gb300")],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-3000:]
    first, second = out.stdout.strip().splitlines()[-2:]
    assert first.startswith("1 True") and "opaque is 8 bytes" in first, first
    assert second.startswith("2 True") and "not a dips_xla_desc_t" in second, second
