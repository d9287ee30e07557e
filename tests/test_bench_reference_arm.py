"""`bench.py --impl reference` runs on CPU. It times the reference's
algorithm (the oracle's C restatement) on the host cores, as independent
replicas. These tests check its JSON line against the bench contract, alone
and under torchrun with two ranks, where rank 0 alone prints and the other
rank exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

from conftest import REPO

BENCH = os.path.join(REPO, "bench.py")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _json_lines(stdout):
    return [json.loads(l) for l in stdout.splitlines() if l.startswith("{")]


def _check_line(line, n_gpus):
    assert line["impl"] == "reference"
    assert line["unit"] == "Gcell-steps/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["n_gpus"] == n_gpus
    assert line["steps"] == 1 and line["warmup"] == 3
    assert line["config"]["workload"] == "cube512"
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_line(oracle_lib):
    out = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr
    lines = _json_lines(out.stdout)
    assert len(lines) == 1
    _check_line(lines[0], 1)


def test_reference_arm_under_torchrun_prints_once(oracle_lib):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), BENCH,
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=REPO, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = _json_lines(out.stdout)
    assert len(lines) == 1
    _check_line(lines[0], 2)
