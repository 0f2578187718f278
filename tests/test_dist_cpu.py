"""Multi-process bench logic on CPU: two gloo ranks on 127.0.0.1 run the
benchmark's own process-group set-up, barrier and max-over-ranks timing,
and the reference arm, where rank 0 alone measures and prints one JSON line
and the other ranks exit without work.  (The data path needs no collective:
the SpMM shards by rows, so N GPUs run N replicas.)"""
import contextlib
import io
import json
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    # CPU ranks wherever the test runs (gloo, no device selection)
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    sys.argv = ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1"]
    import bench
    import torch.distributed as dist
    # a tiny stand-in for the CPU sample (the real one runs for seconds)
    bench.workload = lambda: ({"name": "stand-in", "M": 8}, 1_000_000, (0, 0, 0))
    bench.cpu_sample_rows = lambda cfg, seconds, threads: 8
    bench.cpu_reference = lambda cfg, rows, threads: (0.001, 0.001, "stand-in sample")
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(bench.parse())
    ws = int(os.environ["WORLD_SIZE"])
    bench.barrier(ws)
    m = bench.max_over_ranks(ws, float(rank + 1) * 1.5)
    bench.barrier(ws)
    dist.destroy_process_group()
    q.put((rank, out.getvalue(), m))


def test_two_gloo_ranks_barrier_max_and_reference_arm():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r, out, m = q.get(timeout=180)
        res[r] = (out, m)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # max over ranks reaches every rank
    assert res[0][1] == 3.0 and res[1][1] == 3.0
    # rank 0 prints exactly one line for the reference arm; rank 1 prints nothing
    lines = [l for l in res[0][0].splitlines() if l.strip()]
    assert len(lines) == 1 and res[1][0].strip() == ""
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert abs(line["value"] - 1.0) < 1e-9 and line["e2e"]["h2d_bytes_per_step"] == 0
