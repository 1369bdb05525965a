"""bench.py's reference arm (the CPU port of the reference's path; no GPU
needed) prints one JSON line with the keys the measurement contract names,
and the GPU arm's flags parse."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-its", "4"], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("C2")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["value_serial_gmres"] > 0 and "threads" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_gpu_arm_flags_parse():
    p = subprocess.run([sys.executable, "bench.py", "--help"], cwd=ROOT, capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--skip-variants", "--rods",
                 "--specimens"):
        assert flag in p.stdout, flag


def test_reference_arm_under_torchrun_prints_once():
    """Launched as for N > 1 (torchrun, two ranks, gloo on CPU): rank 0 runs
    and prints the one line, the other rank exits 0 without work."""
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    p = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps",
                        "1", "--warmup", "0", "--cpu-its", "4"], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
