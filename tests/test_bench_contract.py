"""
The reference arm of ``bench.py`` runs on the CPU (the oracle port, no GPU)
and prints one JSON line with the keys the measurement contract needs:
metric, value and unit, the CPU baseline it measured and the end-to-end
record of the same run. Run here on a two-molecule sample.
"""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
         "--warmup", "1", "--cpu-sample", "2"],
        capture_output=True, text=True, timeout=600, cwd=ROOT, check=True,
    ).stdout.strip().splitlines()
    lines = [ln for ln in out if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e", "dtype", "data"):
        assert key in d, key
    assert d["value"] > 0 and d["unit"] == "molecules/s" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
