"""The profile summaries under profiles/ give commands that still run: every
`python bench.py ...` they record parses with the bench's current options, and
every ncu command leaves the GPU clocks alone (host only)."""
import glob
import os
import re
import shlex
import sys

import pytest

from tests.conftest import ROOT

_STOP = {">", ">>", "&&", "||", "|", ";", "2>&1", ")"}


def _lines():
    for f in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        text = open(f).read().replace("\\\n", " ")
        yield f, [ln.strip().strip("`") for ln in text.splitlines()]


def _bench_args(line):
    toks = shlex.split(line)
    i = toks.index("bench.py")
    out = []
    for t in toks[i + 1:]:
        if t in _STOP or t.startswith(">"):
            break
        out.append(t)
    return out


def test_every_summary_records_its_command():
    for f, lines in _lines():
        assert any("bench.py" in ln for ln in lines), f"{os.path.basename(f)} gives no command"


def test_recorded_bench_commands_parse(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    n = 0
    for f, lines in _lines():
        for ln in lines:
            if "python bench.py" not in ln:
                continue
            monkeypatch.setattr(sys, "argv", ["bench.py"] + _bench_args(ln))
            try:
                bench.parse()
            except SystemExit:
                pytest.fail(f"{os.path.basename(f)}: bench options no longer parse: {ln}")
            n += 1
    assert n >= 10


def test_ncu_commands_leave_clocks_alone():
    for f, lines in _lines():
        for ln in lines:
            if re.search(r"(^|&&\s*|;\s*)ncu\s+-", ln):
                assert "--clock-control none" in ln, f"{os.path.basename(f)}: {ln}"
