"""Every command in the ncu summaries under profiles/ runs committed files:
the scripts it names exist in the repository and the benchmark accepts its
arguments; every ncu command keeps the GPU clocks unlocked."""
from __future__ import annotations

import re
import shlex
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _commands():
    for md in sorted((ROOT / "profiles").glob("*.md")):
        for block in re.findall(r"```\n(.*?)```", md.read_text(), flags=re.S):
            text = block.replace("\\\n", " ")
            for line in text.splitlines():
                if line.strip():
                    yield md.name, line.strip()


def test_profile_commands_run_committed_files():
    import bench
    seen = 0
    for name, cmd in _commands():
        words = shlex.split(cmd)
        if words[0] == "ncu":
            assert "--clock-control" in words and words[words.index("--clock-control") + 1] == "none", (name, cmd)
        i = words.index("python")
        script, args = words[i + 1], words[i + 2:]
        assert (ROOT / script).is_file(), (name, script)
        if script == "bench.py":
            bench.make_parser().parse_args(args)
        seen += 1
    assert seen >= 10
