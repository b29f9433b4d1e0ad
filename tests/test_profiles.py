"""Every ncu summary under profiles/ names the command that made it; the
`python bench.py ...` part of each must still parse with bench.py's options
(host code, no GPU)."""
import os
import re
import shlex
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = os.path.join(ROOT, "profiles")


def _bench_commands():
    out = []
    for name in sorted(os.listdir(PROFILES)):
        if not name.endswith(".md"):
            continue
        text = open(os.path.join(PROFILES, name)).read().replace("\\\n", " ")
        for m in re.finditer(r"python bench\.py([^\n`>|&]*)", text):
            out.append((name, m.group(1)))
    return out


def test_profiles_name_their_commands():
    names = [n for n in os.listdir(PROFILES) if n.endswith(".md")]
    assert names
    for n in names:
        text = open(os.path.join(PROFILES, n)).read()
        assert "ncu" in text and "--clock-control none" in text.replace("\\\n", " "), n


@pytest.mark.parametrize("name,args", _bench_commands())
def test_bench_command_parses(monkeypatch, name, args):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py"] + shlex.split(args))
    bench.parse()
