"""bench.py's reference arm runs on the host cores alone, so its JSON line (the
fields every bench.py line carries) is checked here without a GPU, on a small batch."""
import json
import os
import subprocess
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--reads", "500", "--cpu-sample-bp", "1e6"],
                         check=True, capture_output=True, text=True, cwd=ROOT, timeout=600).stdout
    lines = [line for line in out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["metric"] == "read bp aligned/s" and d["unit"] == "read bp/s"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"] and d["config"]["extensions"] > 0 and d["config"]["read_bp"] > 0
    # the reference arm times the CPU implementation only: the product's library is never loaded
    assert not any("libgraphaligner_gb300" in lib for lib in d["repo_libraries_loaded"]), d["repo_libraries_loaded"]
    assert any("libga_oracle" in lib for lib in d["repo_libraries_loaded"])
