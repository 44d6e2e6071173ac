"""bench.py --impl reference: the CPU reference arm (the oracle's FP64
Jacobi-PCG on the host cores, the reference's own OpenNL source being absent)
prints one JSON line with the bench's metric, unit and config, a
cpu_baseline describing the run and an e2e block without host<->device
bytes.  A short window keeps it to a few seconds on the CPU."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line(oracle_mod):
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
         "--window", "0.2", "--drain", "0.3"],
        capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["unit"] == "solves/s" and d["higher_is_better"] is True and d["value"] >= 0.0
    assert d["config"]["workload"].startswith("serving stream")
    assert d["config"]["rel_residual"] == 1e-10 and d["config"]["rel_residual_least_squares"] == 1e-11
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
