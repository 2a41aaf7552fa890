"""The Node-API addon (avbd-sandbox_gb300/napi/avbd_node.cc) compiles against
the C ABI and the Node-API declarations it uses (tests/napi_stub/node_api.h),
with no warnings. Building and running it needs Node.js, absent here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_addon_compiles_cleanly():
    src = os.path.join(ROOT, "avbd-sandbox_gb300", "napi", "avbd_node.cc")
    stub = os.path.join(ROOT, "tests", "napi_stub")
    res = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", stub, src],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
