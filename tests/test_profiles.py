"""The ncu summaries under profiles/ must stay reproducible from committed
files: every script they run exists in the repository, and every bench.py
option they use (--profile-case, --workload) is one bench.py accepts."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench_choices(flag):
    src = (ROOT / "bench.py").read_text()
    m = re.search(r'add_argument\("' + re.escape(flag) + r'",\s*choices=\[([^\]]*)\]', src, re.S)
    assert m, flag
    return set(re.findall(r'"([a-z_0-9]+)"', m.group(1)))


def test_profile_commands_use_committed_files_and_valid_options():
    summaries = sorted((ROOT / "profiles").glob("*.md"))
    assert summaries
    cases, workloads = _bench_choices("--profile-case"), _bench_choices("--workload")
    for md in summaries:
        text = md.read_text()
        assert "python " in text or "ncu " in text, f"{md.name}: no command given"
        for script in re.findall(r"python ([\w./-]+\.py)", text):
            assert (ROOT / script).is_file(), f"{md.name}: {script} is not in the repository"
            assert not script.startswith("_work"), f"{md.name}: runs a working file"
        for case in re.findall(r"--profile-case ([a-z_0-9]+)", text):
            assert case in cases, f"{md.name}: unknown profile case {case}"
        for wl in re.findall(r"--workload ([a-z_0-9]+)", text):
            assert wl in workloads, f"{md.name}: unknown workload {wl}"
