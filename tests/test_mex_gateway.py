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


def test_shims_call_commands_the_gateway_dispatches():
    """Every sid_mex('<command>', ...) in the .m shims names a command the
    gateway's dispatch handles, and every sid_* helper a shim calls is a
    committed .m file or the gateway itself."""
    import glob
    import re
    mdir = os.path.join(ROOT, "sid_gb300", "matlab")
    gateway = open(os.path.join(mdir, "sid_mex.c")).read()
    handled = set(re.findall(r'strcmp\(cmd, "([a-z0-9_]+)"\)', gateway))
    helpers = {os.path.splitext(os.path.basename(f))[0] for f in glob.glob(os.path.join(mdir, "*.m"))}
    called, used_helpers = set(), set()
    for f in glob.glob(os.path.join(mdir, "*.m")):
        text = open(f).read()
        called |= set(re.findall(r"sid_mex\(\s*'([a-z0-9_]+)'", text))
        used_helpers |= set(re.findall(r"\b(sid_[a-z_]+)\s*\(", text)) - {"sid_mex"}
    assert called, "no shim calls the gateway"
    assert called <= handled, called - handled
    assert used_helpers <= helpers, used_helpers - helpers
