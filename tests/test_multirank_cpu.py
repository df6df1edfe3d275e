"""The N>1 path of bench.py on CPU with gloo, world size 2.  The rendering
path has no exchange step (frames and requests are independent: replicas
only), so ranks meet only in the timing barrier and the max-over-ranks
reduction; under torchrun the reference arm runs on rank 0 alone and prints
one JSON line while the other rank exits 0 without work."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    ws, r, _ = bench.dist_setup()
    bench.barrier(ws)
    q.put((r, ws, bench.max_over_ranks(1.5 + r, ws)))
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--workload", "config1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in d, k
    assert d["steps"] == 1 and d["warmup"] == 3 and d["metric"] == d["unit"] == "frames/s"
    assert d["config"]["workload"] and d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]


def test_serving_rows_take_the_median_stream():
    """bench.py's served rows: with several streams per row the reported one
    is the median by frames/s (the lower middle one for an even count), and
    every stream's rate is listed; one stream is reported as it is."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    runs = [{"frames_per_s": 5.0, "p99_ms": 1}, {"frames_per_s": 3.0, "p99_ms": 2}, {"frames_per_s": 9.0, "p99_ms": 3}]
    row = bench._median_run(runs)
    assert row["frames_per_s"] == 5.0 and row["p99_ms"] == 1
    assert row["streams"] == 3 and row["frames_per_s_each"] == [5.0, 3.0, 9.0]
    assert bench._median_run(runs[:2])["frames_per_s"] == 3.0
    assert bench._median_run(runs[:1]) == runs[0]
