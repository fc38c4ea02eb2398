"""The MATLAB MEX gateway (sid_gb300/matlab/sid_mex.c) compiles against the
C ABI (include/sid.h) and minimal declarations of the MEX / mxGPUArray API
(tests/mexstub/): every command's calls into libsid type-check.  MATLAB itself
is not on this machine, so nothing is linked or run."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_mex_gateway_compiles(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = os.path.join(ROOT, "sid_gb300", "matlab", "sid_mex.c")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-Wno-unused-function", "-c", src, "-o",
                        str(tmp_path / "sid_mex.o"), "-I", os.path.join(ROOT, "tests", "mexstub"), "-I",
                        os.path.join(ROOT, "include")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_mex_gateway_calls_only_declared_entry_points():
    import re
    from sid_gb300 import _lib
    text = open(os.path.join(ROOT, "sid_gb300", "matlab", "sid_mex.c")).read()
    used = set(re.findall(r"\b(sid_[a-z0-9_]+)\s*\(", text)) - {"sid_mex"}
    declared = set(_lib.header_functions())
    assert used <= declared, used - declared
