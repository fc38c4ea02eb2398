"""Host-side checks of the per-context cache behind sid_gram_noalloc's scratch
address (sid_gb300/csrc/ctx_cache.h): a value is resolved once per context ID,
a new context ID (after a device reset, or a second context on the same
device) resolves again, and a failed resolution is not kept."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdio>
#include "ctx_cache.h"
int main() {
    sid::CtxCache<long> c;
    int calls = 0;
    long v = 0;
    auto ok = [&](long val) { return [&calls, val](long* o) { ++calls; *o = val; return 0; }; };
    if (c.get(7, ok(100), &v) || v != 100 || calls != 1) return 1;
    if (c.get(7, ok(999), &v) || v != 100 || calls != 1) return 2;   // cached for context 7
    if (c.get(8, ok(200), &v) || v != 200 || calls != 2) return 3;   // a new context resolves again
    if (c.get(7, ok(999), &v) || v != 100 || calls != 2) return 4;   // the old one is still kept
    int rc = c.get(9, [&](long*) { ++calls; return -3; }, &v);
    if (rc != -3 || calls != 3 || c.size() != 2) return 5;           // failures are not cached
    if (c.get(9, ok(300), &v) || v != 300 || calls != 4) return 6;
    std::puts("ok");
    return 0;
}
"""


def test_ctx_cache_keys_by_context(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "t.cpp"
    src.write_text(SRC)
    exe = tmp_path / "t"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "sid_gb300", "csrc"), str(src), "-o",
                    str(exe), "-pthread"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout)
