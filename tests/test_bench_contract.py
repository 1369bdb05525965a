"""bench.py's reference arm (the CPU port of the reference's path; no GPU
needed) prints one JSON line with the keys the measurement contract names,
and the GPU arm's flags parse."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


# bench.py's reference arm run in a process that afterwards reports whether
# the GPU library was ever mapped into it
REF_ARM = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
           "'--warmup', '0']; runpy.run_path('bench.py', run_name='__main__'); "
           "maps = open('/proc/self/maps').read(); "
           "print('GPU-LIBRARY ' + ('MAPPED' if 'libxtfem_gb300' in maps else 'ABSENT'))")


def test_reference_arm_json_line():
    p = subprocess.run([sys.executable, "-c", REF_ARM], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
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
    assert "threads" in cb["sample"] and "stratified" in cb["sample"]
    # a converged solve of the slab, the damage update driven by its solution
    assert d["iterations_per_slab"] > 100 and d["plastic_points"] >= 4
    # the time actually run fits the run: steps x ms_per_step <= wall time
    assert d["steps"] * d["ms_per_step"] <= d["wall_s"] * 1e3
    # the reference arm builds its inputs without the GPU library
    assert "GPU-LIBRARY ABSENT" in p.stdout
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
                        "1", "--warmup", "0"], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
