"""bench.py keeps its one-line JSON contract.  The reference arm (`--impl reference`, the CPU
restatement timed on the host cores) runs here without a GPU; `--quick` shrinks its gate step to
chi = 128 so the test takes seconds."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def test_reference_arm_prints_one_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--quick",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "gate-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "tebd_gate_step_chi128"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "gate-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_a_failing_secondary_leg_keeps_the_line():
    """In a single process a secondary leg that raises is recorded as an error entry, so the
    headline measurement still prints; with several ranks the failure propagates."""
    import importlib.util

    import pytest

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    def boom():
        raise RuntimeError("planted on the host")

    assert bench.guarded("x", lambda: {"ok": 1}, 1) == {"ok": 1}
    assert bench.guarded("x", boom, 1) == {"error": "RuntimeError: planted on the host"}
    with pytest.raises(RuntimeError):
        bench.guarded("x", boom, 2)
