"""The ncu summaries under profiles/ give the commands that produced them;
every bench.py flag those commands use must exist, so the commands stay
runnable as the benchmark changes.  No GPU: only the argument parser is
consulted."""
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_profile_commands_use_existing_bench_flags():
    help_text = subprocess.run([sys.executable, "bench.py", "--help"], cwd=ROOT, capture_output=True, text=True,
                               check=True).stdout
    known = set(re.findall(r"(--[a-z][a-z0-9-]*)", help_text))
    used = set()
    pdir = os.path.join(ROOT, "profiles")
    for fn in os.listdir(pdir):
        txt = open(os.path.join(pdir, fn)).read().replace("\\\n", " ")
        for line in txt.splitlines():
            # direct calls, and calls through a shell variable holding one
            for mark in ("bench.py", "$B "):
                if mark in line:
                    used |= set(re.findall(r"(?<![\w-])(--[a-z][a-z0-9-]*)", line.split(mark, 1)[1]))
    used -= {"--metrics", "--clock-control", "--csv", "--log-file", "--set"}  # ncu's own flags
    assert used, "no bench.py command found under profiles/"
    assert used <= known, sorted(used - known)
