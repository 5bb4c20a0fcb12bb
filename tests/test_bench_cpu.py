"""bench.py's reference arm keeps the benchmark line contract on the host cores (no GPU): one JSON
line with the metric, unit and workload of the GPU arm, a bounded CPU sample described in
``cpu_baseline``, and an ``e2e`` object with no host-device bytes.  Under torchrun with two ranks
rank 0 alone prints it and the other rank exits 0 without work."""

import importlib.util
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, "bench.py")


def _bench_module():
    spec = importlib.util.spec_from_file_location("bench_for_test", BENCH)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _json_lines(text):
    out = []
    for line in text.splitlines():
        line = line.strip()
        if line.startswith("{"):
            out.append(json.loads(line))
    return out


def _check_line(d, n_gpus):
    b = _bench_module()
    argv = sys.argv
    try:
        sys.argv = ["bench.py"]
        args = b.parse()
    finally:
        sys.argv = argv
    assert d["impl"] == "reference"
    assert d["metric"] == b.METRIC and d["unit"] == b.UNIT
    assert d["higher_is_better"] is True and d["n_gpus"] == n_gpus
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == b.nbm_workload(args)
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert "points" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_line():
    p = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = _json_lines(p.stdout)
    assert len(lines) == 1, p.stdout[-2000:]
    _check_line(lines[0], 1)


def test_reference_arm_under_torchrun_prints_once():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), BENCH, "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=900, cwd=ROOT, env=env)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = _json_lines(p.stdout)
    assert len(lines) == 1, p.stdout[-2000:]
    _check_line(lines[0], 2)


def test_algorithmic_flops_per_network_evaluation():
    """The roofline's numerator: F(net) = sum over layers of 2 in out + out, plus one per tanh
    (3 inputs, one output); the training launch counts 3 F per job."""
    b = _bench_module()
    assert b.net_flops(3, 32) == (2 * 3 * 32 + 32) + 2 * (2 * 32 * 32 + 32) + (2 * 32 + 1) + 3 * 32 == 4545
    assert b.net_flops(2, 16) == (2 * 3 * 16 + 16) + (2 * 16 * 16 + 16) + (2 * 16 + 1) + 2 * 16
    assert b.net_flops(4, 64) == (2 * 3 * 64 + 64) + 3 * (2 * 64 * 64 + 64) + (2 * 64 + 1) + 4 * 64
    assert b.net_flops(1, 1) == (2 * 3 + 1) + (2 + 1) + 1
