"""bench.py pieces that run without a GPU: the reference arm (the oracle port
of the reference's CPU path) on the small SIRT workload, alone and under
torchrun with two gloo ranks, the distributed helpers, and the batch
workload's problem generator."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _json_lines(out):
    return [json.loads(x) for x in out.splitlines() if x.startswith("{")]


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload",
                        "sirt256", "--steps", "2", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    (line,) = _json_lines(r.stdout)
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["unit"] == "slice-iter/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["workload"] == bench.WORKLOADS["sirt256"]["name"]


def test_reference_arm_under_torchrun_prints_once():
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
                        "--master-port", str(_free_port()), "bench.py", "--impl",
                        "reference", "--workload", "sirt256", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference"


def _ranks(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2", LOCAL_RANK=str(rank))
    ws, r, _ = bench.dist_setup(0)
    v = bench.max_over_ranks(float(rank + 1), ws)
    bench.barrier(ws)
    q.put((r, ws, v))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_ranks, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    assert got == [(0, 2, 2.0), (1, 2, 2.0)]


def test_batch_problem_generator():
    W = bench.WORKLOADS["batch64"]
    probs = bench.batch_problems(W)
    assert len(probs) == 64
    assert {p["alg"] for p in probs} == {"sirt", "mlem"}
    assert sum(p["alg"] == "sirt" for p in probs) == 32
    assert all(p["C"] in W["widths"] for p in probs)
    assert all(90 <= p["P"] <= 1800 and 1 <= p["S"] <= 16 for p in probs)
    assert probs == bench.batch_problems(W)  # seeded
    for p in probs:
        K = bench.batch_plan_kw(p, type("A", (), {"half": True}))["slices_per_pass"]
        assert K in (1, 2, 4, 8) and K <= max(1, p["S"])
