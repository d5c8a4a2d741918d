"""The bench's command line and the reference arm's JSON line (CPU): the
default run times the whole contour once after three warm-up energies, and
`--impl reference` prints one line with the metric, unit, e2e and
cpu_baseline keys of the contract."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_default_steps_cover_the_contour(monkeypatch):
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    args = b.parse()
    assert args.gpus == 1 and args.warmup >= 3
    e = b.STEP_ENERGIES
    order = [e[i % len(e)] for i in range(args.warmup + args.steps)]
    assert sorted(order[args.warmup:]) == list(range(24))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_reference_arm_of_the_off_diagonal_tau():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "tauij",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"].startswith("(E,k) points/s of the off-diagonal")
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port" and "192 pairs" in line["config"]["workload"]


def test_reference_arm_of_the_three_systems():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c3",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"].startswith("(E,k) points/s of three interface")
    assert line["value"] > 0 and line["config"]["workload"].startswith("c3:")
