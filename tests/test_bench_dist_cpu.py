"""bench.py on the CPU: the multi-rank path with two ranks over gloo (what
torchrun --nproc-per-node 2 sets up, with the GPUs hidden), the max-over-ranks
time and the whole-job rate; the reference arm, which runs on rank 0 only
while the other ranks exit at once without joining a process group; and the
reference arm's JSON line."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r'''
import json, bench
rank, ws, dist = bench.dist_setup()
ms = bench.rank_max(1.5 + rank, dist)          # rank 1 is the slower replica
rate = bench.job_rate(ws, 1000, 10, ms)
print(json.dumps({"rank": rank, "ws": ws, "backend": dist.get_backend(), "ms": ms, "rate": rate}))
dist.barrier()
dist.destroy_process_group()
'''


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, ws, port):
    env = dict(os.environ)
    env.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws), "MASTER_ADDR": "127.0.0.1",
                "MASTER_PORT": str(port), "CUDA_VISIBLE_DEVICES": ""})
    return env


def test_two_gloo_ranks_take_the_slowest_time():
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", WORKER], cwd=ROOT, env=_env(r, 2, port),
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["ws"] == 2 and o["backend"] == "gloo"
        assert o["ms"] == 2.5  # the slower rank's time, on every rank
        assert abs(o["rate"] - 2 * 1000 * 10 / 2.5e-3) < 1e-6 * o["rate"]


def test_reference_arm_runs_on_rank_zero_only():
    port = _free_port()
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "3",
                        "--warmup", "3"], cwd=ROOT, env=_env(1, 2, port), capture_output=True, text=True,
                       timeout=180)
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""


def test_reference_arm_json_line():
    """The reference arm's one JSON line on rank 0 (the oracle on the host
    cores; without a GPU the column is not collapsed first and `sample` says
    so): the keys of the bench contract, with its own cpu_baseline and an e2e
    object that moves no bytes."""
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "1500", "--steps", "3",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.strip().splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config"]:
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0
    assert d["higher_is_better"] is True and d["vs_baseline"] is None and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
