"""The ncu summaries under profiles/: each names the command that made it,
every ncu command leaves the GPU clocks alone, and the commands run only
files of this repository."""
import glob
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = os.path.join(ROOT, "profiles")


def ncu_commands(text):
    return [l.strip() for l in text.splitlines() if l.strip().startswith("ncu ")]


def test_every_summary_gives_its_commands():
    summaries = sorted(glob.glob(os.path.join(PROFILES, "*.md")))
    assert summaries
    for path in summaries:
        cmds = ncu_commands(open(path).read())
        assert cmds, os.path.basename(path)
        for c in cmds:
            name = os.path.basename(path)
            # clocks untouched, and every capture filtered to named kernels or a
            # single-metric launch list
            assert "--clock-control none" in c, name
            assert " -k " in c or "--metrics gpu__time_duration.sum" in c, name
            # the profiled program is one of the repository's own entry points
            prog = c.split(" python ", 1)[1] if " python " in c else ""
            assert re.match(r"(bench\.py|-m pytest tests/)", prog), (name, prog)
            assert "_work" not in c and "/root" not in c, name


def test_json_figures_name_their_source():
    for path in glob.glob(os.path.join(PROFILES, "*.json")):
        d = json.load(open(path))
        assert "--clock-control none" in d["how"], os.path.basename(path)
