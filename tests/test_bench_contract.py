"""The benchmark's command-line contract on CPU: argument parsing, the reference arm's JSON line (the oracle on the
host cores, small workload), and the label and DRAM-traffic tables the GPU line draws on."""
import importlib.util
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, "bench.py")


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_module", BENCH)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_arguments_parse():
    out = subprocess.run([sys.executable, BENCH, "--help"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--arith", "--gs"):
        assert flag in out.stdout
    assert "auto" in out.stdout and "integer" in out.stdout


def test_reference_arm_line():
    out = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--steps", "1", "--warmup", "3",
                          "--workload", "lap2d100"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] >= 3
    assert d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]


def test_labels_and_traffic_tables():
    b = load_bench()
    assert set(b.GS_LABEL) == {"integer", "fma", "tensor"}
    assert set(b.ARITH_LABEL) == {"f64", "pair", "f32"}
    for key in ("lap3d128", "lap3d128_f64", "lap3d128_f64_integer"):
        t = b.committed_traffic(key)
        assert t is not None and set(t) >= {"gs_dot", "gs_update", "spmv"}
        assert all(0.5 < v < 2.0 for v in t.values())
