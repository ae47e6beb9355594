"""CPU check of bench.py's reference arm (`--impl reference`: the reference's CPU path,
timed beside the GPU arm): one JSON line with the bench line's keys, the same metric and
workload as the GPU line, and a positive throughput, on this machine's cores; the arm
loads nothing of the GPU product.  Run on a smaller domain of the same kind (--dims) to
stay quick here."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(built_lib):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--dims", "120x96x40"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "LES cell-steps/s" and d["value"] > 0
    assert d["warmup"] >= 3 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert (d["config"]["im"], d["config"]["jm"], d["config"]["km"]) == (120, 96, 40)
    assert d["single_core"]["cores"] == 1 and d["single_core"]["value"] > 0


def test_reference_arm_loads_no_product_code():
    """The reference arm's imports: the oracle only, never lesgpu or its library."""
    src = open(os.path.join(ROOT, "bench.py")).read()
    body = src[src.index("def run_reference("):src.index("\ndef ", src.index("def run_reference(") + 10)]
    helpers = src[src.index("def oracle_domain("):src.index("def cpu_baseline_sample(")]
    for part in (body, helpers):
        assert "lesgpu" not in part and "scenario(seed" not in part
        assert "import torch" not in part
