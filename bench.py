"""Benchmark of the bitmap SpMM hot path (one JSON line on rank 0).

Workload (default): the clustered plain-FP32 configuration — A 8192×8192
packed bit rows (64 Bernoulli(0.05) prototypes, each row a prototype copy
with p=0.002 flips), B 8192×512 FP32 N(0,1), C = A·B in FP32.  A "step" is
one bitmap-SpMM call over one batch (one B); A's plan (similarity row
grouping) is built once before the timed region, as the reference builds its
row groups before its timed compute (source/src/main.cu:2045 vs :2150-2202);
the plan build time is reported separately and is inside the e2e figure.

Metric: GB/s of compulsory bytes (A packed + B + C) per second.
Timing: CUDA events on the launching stream around K steps replayed from a
CUDA graph; the steps rotate over 8 independent (B, C) pairs, 256 MiB in
total (> the 129 MB L2), so no step finds its inputs in L2.

--impl reference times the reference's CPU path (check()'s dense triple loop,
backup/bit_wise_gemm.cu:13-32, restated in oracle/) on all host threads.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "bitmap-SpMM GB/s (compulsory bytes A+B+C / time)"
UNIT = "GB/s"
ROTATE = 8


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-secondary", action="store_true",
                   help="default run only: skip the compact c1/c3/c4/c4fb/c5 records")
    p.add_argument("--config", default="c2",
                   choices=["c1", "c2", "c3", "c4", "c4fb", "c5", "f1", "f2", "f3", "l2probe"],
                   help="c2 (default): clustered FP32 8192x8192x512; c1: 1024x1024x256 "
                        "integer B; c3: block-structured 16384x16384x2048 BF16 (tensor cores); "
                        "c4: 512 batched problems, N=128 BF16; c4fb: their batched forward+backward; "
                        "c5: forward+backward of a 4096x4096 mask with 4096x8192 BF16 X")
    return p.parse_args()


def dist_setup(args):
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def tensor_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def traffic_from_profiles():
    """DRAM bytes per step from the committed ncu summary (line
    'dram_bytes_per_step: <n>'), or None."""
    path = os.path.join(ROOT, "profiles", "spmm_clustered_8192x8192x512_f32.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_step:"):
            try:
                return int(line.split(":")[1].strip())
            except ValueError:
                return None
    return None


def err_vs_f64(A_bits, B, C):
    """Error of C (rows of A·B) against the same product in FP64, computed
    here with numpy (float64 matmul of the 0/1 rows and B).
    max_scaled / mean_scaled: |C - C64| / (|A||B|)_ij, the scale of the
    summation bound (entries with zero scale must be exact);
    max_rel / mean_rel: elementwise |C - C64| / |C64| over the entries with
    |C64| >= 1e-3 * scale (where a relative error is meaningful)."""
    A64 = np.asarray(A_bits, np.float64)
    B64 = np.asarray(B, np.float64)
    C64 = A64 @ B64
    scale = A64 @ np.abs(B64)
    err = np.abs(np.asarray(C, np.float64) - C64)
    sc = np.where(scale > 0, err / np.where(scale > 0, scale, 1.0), err)
    sel = (np.abs(C64) >= 1e-3 * scale) & (scale > 0)
    rel = err[sel] / np.abs(C64[sel]) if sel.any() else np.zeros(1)
    return {"max_scaled": float(sc.max()), "mean_scaled": float(sc.mean()),
            "max_rel": float(rel.max()), "mean_rel": float(rel.mean()), "entries": int(C64.size)}


def l2_gather_roof(dev, rows=8192, row_bytes=2048):
    """The L2 row-gather roof (bsp_probe_gather): random row slices of a
    16 MB buffer (the size of the clustered step's B, L2-resident) gathered
    by 64 warps per SM, one slice in flight per warp, ~268 MB per launch.
    Returns {slice bytes: GB/s} (best of 5 timed launches each)."""
    import torch
    from bitwise_spgemm_gb300 import capi
    buf = torch.randn(rows * row_bytes // 4, device=dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    n_warps = sms * 64
    out = {}
    for slice_bytes in (512, 1024, 2048):
        per_warp = max(32, (268 << 20) // slice_bytes // n_warps)
        g = torch.Generator(device=dev)
        g.manual_seed(slice_bytes)
        idx = torch.randint(0, rows, (n_warps * per_warp,), device=dev, generator=g, dtype=torch.int64).to(torch.int32)
        sink = torch.zeros(n_warps, device=dev)
        stream = torch.cuda.current_stream(dev)

        def launch():
            capi.call("bsp_probe_gather", buf.data_ptr(), rows, row_bytes, idx.data_ptr(), n_warps, per_warp,
                      slice_bytes, sink.data_ptr(), stream.cuda_stream)
        best = float("inf")
        for i in range(7):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            launch()
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= 2:
                best = min(best, e0.elapsed_time(e1))
        out[slice_bytes] = n_warps * per_warp * slice_bytes / (best * 1e-3) / 1e9
    return out


def run_l2probe(args):
    import torch
    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    roof = l2_gather_roof(dev)
    out = {"metric": "L2 row-gather GB/s (random slices of a 16 MB L2-resident buffer)",
           "value": max(roof.values()), "unit": "GB/s", "n_gpus": ws, "steps": 5, "warmup": 2,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (random rows)", "config": {"workload": "l2_gather_probe_8192x2048B",
                                                        "warps_per_sm": 64, "slices": "one in flight per warp"},
           "by_slice_bytes": {str(k): v for k, v in roof.items()}}
    if rank == 0:
        print(json.dumps(out), flush=True)


def e2e_native(cfg, words_np, B_np, C_ref, args, local, ws, comp_bytes):
    """Runs the C++ end-to-end loop (bsp_e2e) on this rank's GPU, with the
    plan built every step and with the plan reused.  Returns ({reuse: GB/s},
    whether its last C equals C_ref bit for bit, the driver's lines)."""
    import tempfile
    from bitwise_spgemm_gb300 import build as libbuild
    exe = libbuild.E2E if os.path.exists(libbuild.E2E) else libbuild.build_e2e()
    env = dict(os.environ)
    vis = env.get("CUDA_VISIBLE_DEVICES")
    ids = [x for x in vis.split(",") if x.strip()] if vis else None
    env["CUDA_VISIBLE_DEVICES"] = ids[local] if ids and local < len(ids) else str(local)
    out, runs, match = {}, {}, True
    with tempfile.TemporaryDirectory() as d:
        np.ascontiguousarray(words_np).tofile(os.path.join(d, "words.bin"))
        np.ascontiguousarray(B_np, np.float32).tofile(os.path.join(d, "B.bin"))
        M, K, N = cfg["M"], cfg["K"], cfg["N"]
        for mode, key in ((0, False), (1, True), (2, "copies")):
            r = subprocess.run([exe, d, str(M), str(K), str(N), str(args.e2e_steps), "3", str(mode)],
                               capture_output=True, text=True, timeout=600, env=env)
            if r.returncode != 0:
                raise RuntimeError("bsp_e2e failed: " + r.stderr[-400:])
            line = json.loads(r.stdout.strip().splitlines()[-1])
            runs[("built", "reused", "copies_only")[mode]] = line
            ms = max_over_ranks(ws, line["ms_per_step"])
            out[key] = ws * comp_bytes / (ms * 1e-3) / 1e9
            if mode < 2:
                Ch = np.fromfile(os.path.join(d, "C.bin"), np.float32).reshape(M, N)
                match = match and bool(np.array_equal(Ch, C_ref)) and line["device_status"] == 0
    return out, match, runs


def sample_rows(M, n):
    return np.unique(np.linspace(0, M - 1, min(M, n)).astype(np.int64))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def workload():
    from bitwise_spgemm_gb300 import workloads as W
    cfg = W.config2()
    M, K, N = cfg["M"], cfg["K"], cfg["N"]
    bytes_A = M * ((K + 31) // 32) * 4
    bytes_B = K * N * 4
    bytes_C = M * N * 4
    return cfg, bytes_A + bytes_B + bytes_C, (bytes_A, bytes_B, bytes_C)


def cpu_sample_rows(cfg, seconds, threads):
    """Rows of check()'s dense triple loop that `threads` threads finish in
    about `seconds` (calibrated on one row per thread)."""
    import oracle as O
    from bitwise_spgemm_gb300 import workloads as W
    Ad = W.unpack_bits(cfg["words"][:threads], cfg["K"]).astype(np.float32)
    t0 = time.perf_counter()
    O.dense_check_sum(Ad, cfg["B"], threads=threads)
    t_par = time.perf_counter() - t0
    return int(min(cfg["M"], threads * max(1, int(seconds / max(t_par, 1e-6)))))


def cpu_reference(cfg, rows, threads):
    """check()'s triple loop (backup/bit_wise_gemm.cu:13-32, restated in
    oracle/) on the first `rows` rows.  Returns (seconds for those rows,
    seconds scaled to all M rows, description of the sample)."""
    import oracle as O
    from bitwise_spgemm_gb300 import workloads as W
    M, K = cfg["M"], cfg["K"]
    Ad = W.unpack_bits(cfg["words"][:rows], K).astype(np.float32)
    t0 = time.perf_counter()
    O.dense_check_sum(Ad, cfg["B"], threads=threads)
    dt = time.perf_counter() - t0
    return dt, dt * M / rows, ("first %d of %d rows of the dense FP32 triple loop (check(), p ascending) "
                               "on %d thread%s; rate = those rows' share of the compulsory bytes / their time"
                               % (rows, M, threads, "" if threads == 1 else "s"))


def cpu_baselines(cfg, comp_bytes, seconds):
    """The reference's CPU path timed on the host: one core, as the
    reference's loop is serial (the planned baseline), and all host threads
    (a second key).  Each on a row sample of about `seconds` seconds."""
    out = {}
    for key, threads in (("cpu_baseline", 1), ("cpu_baseline_all_threads", os.cpu_count() or 1)):
        rows = cpu_sample_rows(cfg, seconds, threads)
        _, t_full, sample = cpu_reference(cfg, rows, threads)
        out[key] = {"value": comp_bytes / t_full / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
                    "sample": sample}
    return out


def run_reference(args):
    """The reference arm: check()'s triple loop on all host threads.  A step
    is a fixed sample of whole rows (the first R of M), sized so that the
    requested warm-up and timed steps take about a minute together; the
    rate is those rows' share of the compulsory bytes over their time, and
    ms_per_step is the measured time of one such step."""
    ws, rank, _ = dist_setup(args)
    if rank != 0:
        return
    cfg, comp_bytes, _ = workload()
    threads = os.cpu_count() or 1
    per_step = max(0.2, min(5.0, 60.0 / max(1, args.steps + args.warmup)))
    rows = cpu_sample_rows(cfg, per_step, threads)
    times = []
    sample = ""
    for i in range(args.warmup + args.steps):
        t_rows, _, sample = cpu_reference(cfg, rows, threads)
        if i >= args.warmup:
            times.append(t_rows)
    t = float(np.median(times))
    share = comp_bytes * rows / cfg["M"]
    v = share / t / 1e9
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded numpy, clustered-rows generator)",
           "config": {"workload": "clustered_8192x8192x512_f32", "M": 8192, "K": 8192, "N": 512,
                      "step": "the first %d of 8192 rows (%.1f MB of the compulsory bytes)" % (rows, share / 1e6)},
           "impl": "reference",
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_ours(args):
    import torch
    from bitwise_spgemm_gb300 import capi, ops
    ws, rank, local = dist_setup(args)
    cfg, comp_bytes, (bA, bB, bC) = workload()
    M, K, N = cfg["M"], cfg["K"], cfg["N"]
    words_np = np.ascontiguousarray(cfg["words"]).view(np.int32)
    B_np = cfg["B"]
    dev = torch.device("cuda", local)
    words = torch.from_numpy(words_np).to(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan = ops.Plan(words, K)
    torch.cuda.synchronize()
    plan_ms = (time.perf_counter() - t0) * 1e3
    info = plan.info()
    # rotation set: 8 independent B and C buffers (256 MiB > L2)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    Bs = [torch.from_numpy(B_np).to(dev)] + [torch.randn(K, N, device=dev, generator=gen) for _ in range(ROTATE - 1)]
    Cs = [torch.empty(M, N, device=dev) for _ in range(ROTATE)]
    wsb = plan.workspace_bytes(N)
    wsp = torch.empty(max(wsb, 16), dtype=torch.uint8, device=dev)
    kernels_per_step = 2 if info["mode"] == capi.PLAN_PROTO else 1

    def step(i):
        ops.spmm(words, K, Bs[i % ROTATE], plan=plan, out=Cs[i % ROTATE], workspace=wsp)

    for i in range(max(args.warmup, 3)):
        step(i)
    torch.cuda.synchronize()
    # one rotation (8 steps) captured in a graph, plus single-step graphs so
    # that exactly the requested number of steps is timed
    def capture(idx):
        gr = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream(device=dev)
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            with torch.cuda.graph(gr, stream=stream):
                for i in idx:
                    step(i)
        torch.cuda.synchronize()
        return gr

    g = capture(range(ROTATE))
    steps = max(1, args.steps)
    reps, rem = steps // ROTATE, steps % ROTATE
    # the remainder as graphs of 4, 2 and 1 steps (buffers 0.., the 8-step
    # rotation having used them long before)
    g1 = [capture(range(k)) for k in (4, 2, 1) if rem & k]
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    # warm-up right before the timed region (at least 3 rotations, so that a
    # short run is not timed while the clocks come up from the set-up)
    for _ in range(max(3, args.warmup // ROTATE)):
        g.replay()
    for gr in g1:  # a graph's first launch uploads it: keep that out of the timed region
        gr.replay()
    torch.cuda.synchronize()
    # per-rotation timing (one graph of 8 steps per event pair), then the total
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * max(reps, 1))]
    barrier(ws)
    torch.cuda.synchronize()
    cur = torch.cuda.current_stream()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(cur)
    for r in range(reps):
        ev[2 * r].record(cur)
        g.replay()
        ev[2 * r + 1].record(cur)
    for gr in g1:
        gr.replay()
    t_end.record(cur)
    torch.cuda.synchronize()
    barrier(ws)
    clocks = sampler.stop() if sampler else None
    total_ms = t_start.elapsed_time(t_end)
    total_ms = max_over_ranks(ws, total_ms)
    ms_step = total_ms / steps
    value = ws * comp_bytes / (ms_step * 1e-3) / 1e9
    launch_ms = (float(np.mean([ev[2 * r].elapsed_time(ev[2 * r + 1]) for r in range(reps)])) / ROTATE
                 if reps else ms_step)

    # correctness spot check of the last rotation against a direct walk, and
    # the error against FP64 on a row sample
    Cd = ops.spmm(words, K, Bs[0])
    torch.cuda.synchronize()
    err = (Cs[0] - Cd).abs().max().item() / max(Cd.abs().max().item(), 1e-30)
    from bitwise_spgemm_gb300 import workloads as W
    rows = sample_rows(M, 256)
    err64 = err_vs_f64(W.unpack_bits(cfg["words"][rows], K), B_np, Cs[0].cpu().numpy()[rows])
    err64["sample"] = "%d rows evenly spaced over %d" % (len(rows), M)

    # e2e through the C ABI from a C++ serving loop (harness/bsp_e2e): pinned
    # host A words and B in, plan, SpMM, C out, per step, two steps in
    # flight; once with the plan built every step, once reused
    e2e, e2e_matches, e2e_runs = e2e_native(cfg, words_np, B_np, Cs[0].cpu().numpy(), args, local, ws, comp_bytes)

    peak, peak_kind = peaks()
    achieved = comp_bytes / (launch_ms * 1e-3) / 1e9
    # the step's L2 gathers: prototype bits and delta entries (one B row
    # each), one prototype-sum row read per clustered row
    l2_bytes = (info["proto_nnz"] + info["delta_nnz"] + info["direct_nnz"] + M) * N * 4
    roof = l2_gather_roof(dev)
    traffic = traffic_from_profiles()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy clustered-rows A, N(0,1) B; 7 further random B in the rotation)",
        "config": {"workload": "clustered_8192x8192x512_f32", "M": M, "K": K, "N": N,
                   "l2": "inputs larger than L2: 8 rotating (B, C) pairs, 256 MiB",
                   "plan_mode": "proto" if info["mode"] == capi.PLAN_PROTO else "direct",
                   "plan_ms": plan_ms, "n_proto": info["n_proto"], "delta_nnz": info["delta_nnz"],
                   "nnz": info["nnz"], "direct_rows": info["direct_rows"],
                   "graph": "CUDA graphs of 8 steps (and of 4, 2, 1 for the remainder), replayed after a warm-up replay each"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind,
                     "units": "compulsory bytes of one SpMM call (proto sums + row kernel)",
                     "l2_gather": {"achieved": l2_bytes / (launch_ms * 1e-3) / 1e9,
                                   "peak": max(roof.values()),
                                   "frac": l2_bytes / (launch_ms * 1e-3) / 1e9 / max(roof.values()),
                                   "unit": "GB/s", "bytes_per_step": l2_bytes,
                                   "peak_source": "bsp_probe_gather in this run (best slice size)",
                                   "probe_by_slice_bytes": {str(k): v for k, v in roof.items()}}},
        "e2e": {"value": e2e[True], "unit": UNIT, "h2d_bytes_per_step": bA + bB,
                "d2h_bytes_per_step": bC,
                "includes": "H2D A words + B, SpMM, D2H C every step; A's plan built once before the timed "
                            "steps, as for value (the reference builds its groups before its timed compute)",
                "pipeline": "two steps in flight: step i's D2H overlaps step i+1's uploads",
                "plan_per_step_value": e2e[False],
                "caller": "C++ serving loop through the C ABI (bitwise_spgemm_gb300/harness/bsp_e2e.cpp), "
                          "wall clock over %d steps" % args.e2e_steps,
                "link_roof": {"value": e2e["copies"], "unit": UNIT,
                              "what": "the same loop's uploads and downloads alone (no plan, no SpMM)",
                              "frac_plan_built": e2e[False] / e2e["copies"],
                              "frac_plan_reused": e2e[True] / e2e["copies"]},
                "runs": e2e_runs},
        "gpu_launches": steps * kernels_per_step,
        "clocks": clocks,
        "max_rel_diff_vs_direct": err,
        "error_vs_fp64": err64,
        "e2e_output_matches_graph_output": e2e_matches,
    }
    if rank == 0:
        out["cusparse"] = _cusparse(words, K, Bs[0], launch_ms, Cd)
    if rank == 0 and ws == 1 and not args.no_cpu:
        out.update(cpu_baselines(cfg, comp_bytes, args.cpu_seconds))
    plan.close()
    if rank == 0 and ws == 1 and not args.no_secondary:
        out["secondary"] = secondary(args, dev)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_other(args, config=None, emit=True):
    """Secondary configurations: c1 (plain small, integer B) and c3 (block-
    structured, BF16 B on the tensor cores).  Same timing rules: CUDA events
    on the launching stream around K steps, warm-up first."""
    import torch
    from bitwise_spgemm_gb300 import capi, ops
    from bitwise_spgemm_gb300 import workloads as W
    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    config = config or args.config
    cfg = W.config1() if config == "c1" else W.config3()
    M, K, N = cfg["M"], cfg["K"], cfg["N"]
    words = torch.from_numpy(np.ascontiguousarray(cfg["words"]).view(np.int32)).to(dev)
    if cfg["b_dtype"] == "bf16":
        B = torch.from_numpy(np.ascontiguousarray(cfg["B"]).view(np.int16)).to(dev).view(torch.bfloat16)
        esz, dtype = 2, "bf16"
    else:
        B = torch.from_numpy(cfg["B"]).to(dev)
        esz, dtype = 4, "f32"
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan = ops.Plan(words, K)
    torch.cuda.synchronize()
    plan_ms = (time.perf_counter() - t0) * 1e3
    info = plan.info()
    C = torch.empty(M, N, device=dev)
    wsp = torch.empty(max(plan.workspace_bytes(N), 16), dtype=torch.uint8, device=dev)
    comp = M * ((K + 31) // 32) * 4 + K * N * esz + M * N * 4
    flops = 2.0 * info["nnz"] * N

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cur = torch.cuda.current_stream()
        e0.record(cur)
        for _ in range(steps):
            fn()
        e1.record(cur)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    step = lambda: ops.spmm(words, K, B, plan=plan, out=C, workspace=wsp)
    # the step replayed from a CUDA graph (no host launch cost in the time)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    # 8 steps per graph, so that a short step is not timed at the host's
    # replay rate
    per_graph = 8
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            for _ in range(per_graph):
                step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    barrier(ws)
    reps = max(1, (args.steps + per_graph - 1) // per_graph)
    ms = max_over_ranks(ws, timed(graph.replay, reps, max(1, args.warmup // per_graph)) / per_graph)
    barrier(ws)
    clocks = sampler.stop() if sampler else None
    # error against FP64: every row of c1 (integer B: must be exact), a row
    # sample of c3
    Bh = cfg["B"] if cfg["b_dtype"] != "bf16" else W.bf16_bits_to_f32(cfg["B"])
    rows = np.arange(M) if config == "c1" else sample_rows(M, 64)
    err64 = err_vs_f64(W.unpack_bits(cfg["words"][rows], K), Bh, C.cpu().numpy()[rows])
    err64["sample"] = "all %d rows" % M if config == "c1" else "%d rows evenly spaced over %d" % (len(rows), M)
    out = {"metric": METRIC, "value": ws * comp / (ms * 1e-3) / 1e9, "unit": UNIT, "n_gpus": ws,
           "steps": reps * per_graph, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded numpy)",
           "config": {"workload": cfg["name"], "M": M, "K": K, "N": N, "plan_ms": plan_ms,
                      "nnz": info["nnz"], "l2": "working set %.0f MB" % (comp / 1e6),
                      "graph": "8 steps per CUDA graph, replayed (steps rounded up to whole graphs)"},
           "effective_gflops": flops / (ms * 1e-3) / 1e9, "error_vs_fp64": err64, "clocks": clocks}
    if config == "c3":
        occ = info["occ_tiles"]
        dense = occ * 128 * 32 * N * 2.0
        tp, tkind = tensor_peak()
        out["tensor"] = {"issued_tflops": dense / (ms * 1e-3) / 1e12, "peak_tflops": tp,
                         "frac": dense / (ms * 1e-3) / 1e12 / tp, "peak_source": tkind,
                         "occupied_tiles": occ}
        # the same problem in the plain FP32 form (CUDA cores): a few steps
        Bf = torch.from_numpy(W.bf16_bits_to_f32(cfg["B"])).to(dev)
        step32 = lambda: ops.spmm(words, K, Bf, plan=plan, out=C, workspace=wsp)
        ms32 = timed(step32, 2, 1)
        out["fp32_form_ms"] = ms32
        out["speedup_vs_fp32_form"] = ms32 / ms
        step()
    if rank == 0 and emit:
        out["cusparse"] = _cusparse(words, K, B, ms, C, iters=3)
        print(json.dumps(out), flush=True)
    plan.close()
    return out


def run_batched(args, emit=True):
    """Batched form: 512 independent problems (M, K log-uniform in [64, 4096],
    density U(0.01, 0.3), N = 128, BF16 B) in one persistent graph-captured
    launch, against looping the plain FP32 single-problem SpMM (also
    graph-captured, so host launch overhead counts for neither)."""
    import torch
    from bitwise_spgemm_gb300 import capi, ops
    from bitwise_spgemm_gb300 import workloads as W
    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    probs = W.config4()
    N = 128
    items, items32 = [], []
    comp = 0
    nnz = 0
    for pr in probs:
        M, K = pr["M"], pr["K"]
        wd = torch.from_numpy(np.ascontiguousarray(pr["words"]).view(np.int32)).to(dev)
        B = torch.from_numpy(pr["B"].view(np.int16)).to(dev).view(torch.bfloat16)
        items.append((wd, K, B, torch.empty(M, N, device=dev)))
        items32.append((wd, K, B.float(), torch.empty(M, N, device=dev)))
        comp += M * ((K + 31) // 32) * 4 + K * N * 2 + M * N * 4
        nnz += int(np.unpackbits(np.ascontiguousarray(pr["words"]).view(np.uint8)).sum())
    batch = ops.Batch(items)
    # the batch's own tuner picks the persistent kernel's shape (before capture)
    shape, tune_ms = batch.tune()

    def graph_of(fn):
        fn()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        st = torch.cuda.Stream(device=dev)
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            with torch.cuda.graph(g, stream=st):
                fn()
        torch.cuda.synchronize()
        return g

    def loop32():
        for wd, K, B32, Cd in items32:
            ops.spmm(wd, K, B32, out=Cd)

    gb = graph_of(batch.run)
    g32 = graph_of(loop32)

    def timed(g, steps, warm):
        for _ in range(warm):
            g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cur = torch.cuda.current_stream()
        e0.record(cur)
        for _ in range(steps):
            g.replay()
        e1.record(cur)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    barrier(ws)
    ms = max_over_ranks(ws, timed(gb, args.steps, max(args.warmup, 3)))
    barrier(ws)
    clocks = sampler.stop() if sampler else None
    ms32 = timed(g32, 3, 1)
    # spot check against the FP32 loop, and the error against FP64 on every
    # 16th problem
    err = max(float((a[3] - b[3]).abs().max()) / max(float(b[3].abs().max()), 1e-30)
              for a, b in zip(items[:8], items32[:8]))
    errs = [err_vs_f64(W.unpack_bits(probs[i]["words"], probs[i]["K"]), W.bf16_bits_to_f32(probs[i]["B"]),
                       items[i][3].cpu().numpy()) for i in range(0, len(probs), 16)]
    err64 = {k: (max if k.startswith("max") else np.mean)([e[k] for e in errs]) for k in errs[0] if k != "entries"}
    err64 = {k: float(v) for k, v in err64.items()}
    err64["sample"] = "every 16th problem (%d of %d), all rows" % (len(errs), len(probs))
    out = {"metric": "batched bitmap-SpMM problems/s", "value": ws * len(probs) / (ms * 1e-3),
           "unit": "problems/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16", "data": "synthetic (seeded numpy, seed 7+i per problem)",
           "config": {"workload": "batched_512_N128_bf16", "problems": len(probs), "N": N,
                      "nnz": nnz, "graph": "one persistent launch (a CTA per SM taking 256-row items from a device work queue), graph-captured",
                      "kernel_shape": {"index": shape, "tuned_ms": tune_ms,
                                       "by": "bsp_batch_tune (stages, epilogue warps, A words ahead)"}},
           "aggregate_gbs": ws * comp / (ms * 1e-3) / 1e9,
           "effective_tflops": 2.0 * nnz * N / (ms * 1e-3) / 1e12,
           "fp32_loop_ms": ms32, "speedup_vs_fp32_loop": ms32 / ms,
           "max_rel_diff_vs_fp32_loop": err, "error_vs_fp64": err64, "clocks": clocks}
    if rank == 0 and emit:
        print(json.dumps(out), flush=True)
    batch.close()
    return out


def run_batched_fb(args, emit=True):
    """Batched forward+backward: for the 512 problems of the batched set
    (A_i, X_i = B_i BF16, N = 128) and a seeded incoming gradient G_i, the
    BF16 batched form computes Y_i = A_i·X_i (persistent batched kernel),
    dX_i = A_iᵀ·G_i and dA_i = (G_i·X_iᵀ) ⊙ A_i (batched tensor-core
    launches), all in one CUDA graph.  It is timed against the plain FP32
    per-problem form: a graph-captured loop of bsp_spmm, bsp_spmm_t and
    bsp_sddmm on FP32 copies of the same operands (CUDA cores)."""
    import torch
    from bitwise_spgemm_gb300 import ops
    from bitwise_spgemm_gb300 import workloads as W
    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    probs = W.config4()
    N = 128
    fwd, grad, loop32 = [], [], []
    G16s = []
    nnz = 0
    for i, pr in enumerate(probs):
        M, K = pr["M"], pr["K"]
        wd = torch.from_numpy(np.ascontiguousarray(pr["words"]).view(np.int32)).to(dev)
        X = torch.from_numpy(pr["B"].view(np.int16)).to(dev).view(torch.bfloat16)
        g16 = W.config4_grad(pr, i)
        G16s.append(g16)
        G = torch.from_numpy(g16.view(np.int16)).to(dev).view(torch.bfloat16)
        Y, dX, dA = (torch.empty(M, N, device=dev), torch.empty(K, N, device=dev), torch.empty(M, K, device=dev))
        fwd.append((wd, K, X, Y))
        grad.append((wd, K, X, G, dX, dA))
        loop32.append((wd, M, K, X.float(), G.float(), torch.empty(M, N, device=dev), torch.empty(K, N, device=dev),
                       torch.empty(M, K, device=dev)))
        nnz += int(np.unpackbits(np.ascontiguousarray(pr["words"]).view(np.uint8)).sum())
    bf = ops.Batch(fwd)
    bg = ops.BatchGrad(grad)
    # one workspace for the FP32 transposed products (the calls run in order)
    import ctypes
    from bitwise_spgemm_gb300 import capi
    need = 0
    for wd, M, K, *_ in loop32:
        n = ctypes.c_size_t()
        capi.call("bsp_spmm_t_workspace_preferred", M, K, N, ctypes.byref(n))
        need = max(need, n.value)
    wsp = torch.empty(max(need, 16), dtype=torch.uint8, device=dev)

    def step16():
        bf.run()
        bg.run()

    def step32():
        for wd, M, K, X32, G32, Y32, dX32, dA32 in loop32:
            ops.spmm(wd, K, X32, out=Y32)
            ops.spmm_t(wd, M, K, G32, out=dX32, workspace=wsp)
            ops.sddmm(wd, M, K, G32, X32, out=dA32)

    def graph_of(fn):
        fn()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        st = torch.cuda.Stream(device=dev)
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            with torch.cuda.graph(g, stream=st):
                fn()
        torch.cuda.synchronize()
        return g

    g16, g32 = graph_of(step16), graph_of(step32)
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    barrier(ws)
    ms = max_over_ranks(ws, _timed(g16.replay, max(1, args.steps), max(args.warmup, 3)))
    barrier(ws)
    clocks = sampler.stop() if sampler else None
    ms32 = _timed(g32.replay, 2, 1)
    g16.replay()
    torch.cuda.synchronize()
    # errors against FP64 on every 16th problem: Y and dX all rows, dA at A's bits
    ey, ex, ea = [], [], []
    for i in range(0, len(probs), 16):
        pr = probs[i]
        A = W.unpack_bits(pr["words"], pr["K"])
        X, G = W.bf16_bits_to_f32(pr["B"]), W.bf16_bits_to_f32(G16s[i])
        ey.append(err_vs_f64(A, X, fwd[i][3].cpu().numpy()))
        ex.append(err_vs_f64(A.T, G, grad[i][4].cpu().numpy()))
        dA = grad[i][5].cpu().numpy()
        dA64 = G.astype(np.float64) @ X.astype(np.float64).T
        sc = np.abs(G).astype(np.float64) @ np.abs(X).astype(np.float64).T
        e = np.abs(dA[A] - dA64[A])
        sel = (np.abs(dA64[A]) >= 1e-3 * sc[A]) & (sc[A] > 0)
        ea.append({"max_scaled": float((e / np.maximum(sc[A], 1e-300)).max()) if e.size else 0.0,
                   "max_rel": float((e[sel] / np.abs(dA64[A][sel])).max()) if sel.any() else 0.0,
                   "mean_rel": float((e[sel] / np.abs(dA64[A][sel])).mean()) if sel.any() else 0.0,
                   "off_bits_zero": bool(np.all(dA[~A] == 0.0))})
    summ = lambda L: {"max_scaled": max(e["max_scaled"] for e in L), "max_rel": max(e["max_rel"] for e in L),  # noqa: E731
                      "mean_rel": float(np.mean([e["mean_rel"] for e in L]))}
    err64 = {"Y": summ(ey), "dX": summ(ex), "dA": dict(summ(ea), off_bits_zero=all(e["off_bits_zero"] for e in ea)),
             "sample": "every 16th problem (%d of %d)" % (len(ey), len(probs))}
    max_rel = max(err64[k]["max_rel"] for k in ("Y", "dX", "dA"))
    out = {"metric": "batched bitmap-SpMM forward+backward problems/s (Y, dX, dA)",
           "value": ws * len(probs) / (ms * 1e-3), "unit": "problems/s", "n_gpus": ws, "steps": max(1, args.steps),
           "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded numpy, seed 7+i per problem, G seed 100007+i)",
           "config": {"workload": "batched_512_N128_fwd_bwd_bf16", "problems": len(probs), "N": N, "nnz": nnz,
                      "graph": "one graph: persistent forward launch + batched Aᵀ·G and SDDMM launches"},
           "effective_tflops": 3 * 2.0 * nnz * N / (ms * 1e-3) / 1e12,
           "fp32_loop_ms": ms32, "speedup_vs_fp32_form": ms32 / ms,
           "target": {"speedup_min": 2.0, "max_rel_err_max": 1e-2,
                      "met": bool(ms32 / ms >= 2.0 and max_rel <= 1e-2)},
           "error_vs_fp64": err64, "clocks": clocks}
    if rank == 0 and emit:
        print(json.dumps(out), flush=True)
    bf.close()
    bg.close()
    return out


def secondary(args, dev):
    """Compact records of the other configurations, measured in the same run
    as the headline line so that they are observed by whoever runs it: the
    small plain SpMM (c1), the tensor-core precision form (c3), the batched
    form (c4), the batched forward+backward form (c4fb) and the
    differentiable form (c5)."""
    import copy
    import torch
    a2 = copy.copy(args)
    a2.steps = min(args.steps, 24)
    a2.warmup = 3
    runs = (("c1", lambda: run_other(a2, "c1", emit=False)), ("c3", lambda: run_other(a2, "c3", emit=False)),
            ("c4", lambda: run_batched(a2, emit=False)), ("c4fb", lambda: run_batched_fb(a2, emit=False)),
            ("c5", lambda: run_fwd_bwd(a2, emit=False)))
    sub = {}
    for name, fn in runs:
        t0 = time.perf_counter()
        try:
            o = fn()
        except Exception as exc:  # a failing sub-record must not lose the headline line
            sub[name] = {"error": repr(exc)[:300]}
            continue
        r = {"workload": o["config"]["workload"], "metric": o["metric"], "value": o["value"], "unit": o["unit"],
             "ms_per_step": o["ms_per_step"], "steps": o["steps"], "dtype": o["dtype"],
             "error_vs_fp64": o.get("error_vs_fp64"), "clocks": o.get("clocks")}
        for k in ("speedup_vs_fp32_form", "speedup_vs_fp32_loop", "fp32_form_ms", "fp32_loop_ms", "target",
                  "effective_gflops", "effective_tflops", "aggregate_gbs"):
            if k in o:
                r[k] = o[k]
        if "tensor" in o:
            r["tensor_frac"] = o["tensor"]["frac"]
        r["wall_s"] = time.perf_counter() - t0
        sub[name] = r
        torch.cuda.empty_cache()
    return sub


def run_fwd_bwd(args, emit=True):
    """Differentiable form: Y = A·X, dX = Aᵀ·G, dA = (G·Xᵀ) ⊙ A with A a
    4096x4096 Bernoulli(0.1) mask, X and G 4096x8192 BF16; the same three
    products in the plain FP32 form (CUDA cores) are timed for the speedup."""
    import torch
    from bitwise_spgemm_gb300 import capi, ops
    from bitwise_spgemm_gb300 import workloads as W
    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    cfg = W.config5()
    M, K, N = cfg["M"], cfg["K"], cfg["N"]
    words = torch.from_numpy(np.ascontiguousarray(cfg["words"]).view(np.int32)).to(dev)
    X = torch.from_numpy(cfg["X"].view(np.int16)).to(dev).view(torch.bfloat16)
    G = torch.from_numpy(cfg["G"].view(np.int16)).to(dev).view(torch.bfloat16)
    plan = ops.Plan(words, K)
    info = plan.info()
    Y = torch.empty(M, N, device=dev)
    dX = torch.empty(K, N, device=dev)
    dA = torch.empty(M, K, device=dev)
    wsp = torch.empty(max(plan.workspace_bytes(N), 16), dtype=torch.uint8, device=dev)

    def step16():
        ops.spmm(words, K, X, plan=plan, out=Y, workspace=wsp)
        ops.spmm_t(words, M, K, G, plan=plan, out=dX)
        ops.sddmm(words, M, K, G, X, plan=plan, out=dA)

    X32, G32 = X.float(), G.float()

    def step32():
        ops.spmm(words, K, X32, plan=plan, out=Y, workspace=wsp)
        ops.spmm_t(words, M, K, G32, plan=plan, out=dX)
        ops.sddmm(words, M, K, G32, X32, plan=plan, out=dA)

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cur = torch.cuda.current_stream()
        e0.record(cur)
        for _ in range(steps):
            fn()
        e1.record(cur)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    barrier(ws)
    ms = max_over_ranks(ws, timed(step16, args.steps, max(args.warmup, 3)))
    barrier(ws)
    clocks = sampler.stop() if sampler else None
    step16()
    torch.cuda.synchronize()
    # errors against FP64 on samples: 64 rows of Y, 64 rows of dX (columns
    # of A), the set bits of 64 rows of dA
    A = W.unpack_bits(cfg["words"], K)
    Xh, Gh = W.bf16_bits_to_f32(cfg["X"]), W.bf16_bits_to_f32(cfg["G"])
    rs, ks = sample_rows(M, 64), sample_rows(K, 64)
    ey = err_vs_f64(A[rs], Xh, Y.cpu().numpy()[rs])
    ex = err_vs_f64(A[:, ks].T, Gh, dX.cpu().numpy()[ks])
    dA_rows = dA.cpu().numpy()[rs]
    dA64 = Gh[rs].astype(np.float64) @ Xh.astype(np.float64).T
    dAsc = np.abs(Gh[rs]).astype(np.float64) @ np.abs(Xh).astype(np.float64).T
    m = A[rs]
    e = np.abs(dA_rows[m] - dA64[m])
    sel = (np.abs(dA64[m]) >= 1e-3 * dAsc[m]) & (dAsc[m] > 0)
    ea = {"max_scaled": float((e / np.maximum(dAsc[m], 1e-300)).max()),
          "mean_scaled": float((e / np.maximum(dAsc[m], 1e-300)).mean()),
          "max_rel": float((e[sel] / np.abs(dA64[m][sel])).max()),
          "mean_rel": float((e[sel] / np.abs(dA64[m][sel])).mean()),
          "off_bits_zero": bool(np.all(dA_rows[~m] == 0.0))}
    err64 = {"Y": ey, "dX": ex, "dA": ea, "sample": "64 rows of Y and dA, 64 rows of dX, evenly spaced"}
    ms32 = timed(step32, 2, 1)
    nnz = info["nnz"]
    useful = 3 * 2.0 * nnz * N
    dense = 3 * 2.0 * M * K * N
    tp, tkind = tensor_peak()
    comp = 2 * (M * ((K + 31) // 32) * 4) + 2 * K * N * 2 + 2 * M * N * 2 + M * N * 4 + K * N * 4 + M * K * 4
    out = {"metric": "bitmap-SpMM forward+backward ms (Y, dX, dA)", "value": ms, "unit": "ms",
           "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
           "data": "synthetic (seeded numpy)",
           "config": {"workload": "mask_4096x4096_x_4096x8192_fwd_bwd_bf16", "M": M, "K": K, "N": N,
                      "nnz": nnz},
           "fp32_form_ms": ms32, "speedup_vs_fp32_form": ms32 / ms,
           "effective_tflops": useful / (ms * 1e-3) / 1e12,
           "tensor": {"dense_tflops": dense / (ms * 1e-3) / 1e12, "peak_tflops": tp,
                      "frac": dense / (ms * 1e-3) / 1e12 / tp, "peak_source": tkind},
           "gbs_compulsory": comp / (ms * 1e-3) / 1e9, "error_vs_fp64": err64, "clocks": clocks}
    if rank == 0 and emit:
        # cuSPARSE on the forward product Y = A·X (its SpMM has no fused
        # transposed-bitmap or SDDMM counterpart here)
        ms_fwd = _timed(lambda: ops.spmm(words, K, X, plan=plan, out=Y, workspace=wsp), 5, 2)
        out["cusparse_forward"] = dict(_cusparse(words, K, X, ms_fwd, Y, iters=3), ours_forward_ms=ms_fwd)
        print(json.dumps(out), flush=True)
    plan.close()
    return out


def _timed(fn, steps, warm):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cur = torch.cuda.current_stream()
    e0.record(cur)
    for _ in range(steps):
        fn()
    e1.record(cur)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _cusparse(words, K, B, ours_ms, ours_C, iters=5):
    """cuSPARSE's CSR SpMM on the same A (values 1) and B: the reference's
    library baseline (source/src/main.cu:1061-1131), outside every timed
    region of this benchmark.  `ms` is the warm mean over `iters` calls,
    `first_call_ms` the reference's own measure (workspace query + allocation
    + one call).  Any failure becomes an `unavailable` entry."""
    import torch
    from bitwise_spgemm_gb300 import cusparse_baseline as CS
    ok, why = CS.available()
    if not ok:
        return {"unavailable": why}
    try:
        off, cols = CS.csr_from_words(words, K)
        C, ms, first = CS.spmm_csr(off, cols, B, words.shape[0], warmup=2, iters=iters)
        torch.cuda.synchronize()
        diff = (C - ours_C).abs().max().item() / max(ours_C.abs().max().item(), 1e-30)
        del off, cols, C
        return {"ms": ms, "first_call_ms": first, "alg": "CUSPARSE_SPMM_ALG_DEFAULT, CSR int32, values 1",
                "dtype": "f32" if B.dtype == torch.float32 else "bf16 in, f32 out",
                "speedup_ours_vs_cusparse": ms / ours_ms, "max_rel_diff_vs_ours": diff}
    except (RuntimeError, ValueError) as exc:
        return {"unavailable": str(exc)}


def _cpu_rows(fn, M, rows0=64, budget=5.0):
    """Seconds per full problem of a row-sliced oracle call, from the largest
    row sample (doubling from rows0) that stays within the budget."""
    rows = rows0
    while True:
        t0 = time.perf_counter()
        fn(rows)
        dt = time.perf_counter() - t0
        if dt > budget / 4 or rows >= M:
            return dt * M / rows, rows
        rows = min(M, rows * 2)


def run_next(args):
    """The rows after the SpMM: f1 symbolic output masks + first-fit grouping
    of the output rows, f2 bit-plane int8 product, f3 8x8 bitmap tiles and
    tiled CSR.  One JSON line each; inputs resident, L2 flushed by the size of
    the inputs where they exceed it (stated per workload)."""
    import torch
    import oracle as O
    from bitwise_spgemm_gb300 import ops
    from bitwise_spgemm_gb300 import workloads as W
    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    hbm, hkind = peaks()
    steps, warm = args.steps, max(args.warmup, 3)
    sampler = ClockSampler(local) if rank == 0 else None
    base = {"n_gpus": ws, "steps": steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "data": "synthetic (seeded numpy)"}
    if args.config == "f1":
        cfg = W.config_symbolic()
        M, K, N = cfg["M"], cfg["K"], cfg["N"]
        a = torch.from_numpy(cfg["a_words"].view(np.int32)).to(dev)
        b = torch.from_numpy(cfg["b_words"].view(np.int32)).to(dev)
        out = torch.empty(M, (N + 31) // 32, dtype=torch.int32, device=dev)
        out_walk = torch.empty_like(out)
        # the plan of A (built once, before the timed region, as for the SpMM)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan = ops.Plan(a, K)
        torch.cuda.synchronize()
        plan_ms = (time.perf_counter() - t0) * 1e3
        pinfo = plan.info()
        wsp = ops._ws("bsp_symbolic_workspace", plan._h, N, device=dev)
        step = lambda: ops.symbolic_rows(a, K, b, N, out=out, plan=plan, workspace=wsp)
        step_walk = lambda: ops.symbolic_rows(a, K, b, N, out=out_walk)
        if sampler:
            sampler.start()
        barrier(ws)
        ms = max_over_ranks(ws, _timed(step, steps, warm))
        barrier(ws)
        clocks = sampler.stop() if sampler else None
        ms_walk = _timed(step_walk, max(3, steps // 4), 2)
        same = bool(torch.equal(out, out_walk))
        ms_group = _timed(lambda: ops.group_rows(out, 512, 2), 3, 1)
        nnz = int(np.unpackbits(cfg["a_words"].view(np.uint8)).sum())
        comp = 3 * M * ((N + 31) // 32) * 4
        gather = nnz * ((N + 31) // 32) * 4
        sec, rows = _cpu_rows(lambda r: O.symbolic_rows(cfg["a_words"][:r], K, cfg["b_words"], N), M)
        line = dict(base, metric="symbolic output mask GB/s (A+B+C words / time)", value=comp / (ms * 1e-3) / 1e9,
                    unit="GB/s", ms_per_step=ms, dtype="u32",
                    config={"workload": cfg["name"], "M": M, "K": K, "N": N, "nnz_A": nnz,
                            "plan": "prototype plan of A built before the timed region (plan_ms)",
                            "plan_ms": plan_ms, "n_proto": pinfo["n_proto"], "delta_nnz": pinfo["delta_nnz"],
                            "l2": "B's words (8 MiB) stay in L2; the gathers are L2 reads"},
                    walk_ms=ms_walk, walk_gather_gbs=gather / (ms_walk * 1e-3) / 1e9,
                    speedup_vs_walk=ms_walk / ms, planned_equals_walk=same, grouping_ms=ms_group,
                    roofline={"bound": "hbm", "achieved": comp / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                              "frac": comp / (ms * 1e-3) / 1e9 / hbm, "traffic": None, "peak_source": hkind},
                    cpu_baseline={"value": comp / sec / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                                  "sample": "oracle symbolic pass on the first %d rows, scaled to %d" % (rows, M)},
                    clocks=clocks)
        plan.close()
    elif args.config == "f2":
        cfg = W.config_int8()
        M, K, N = cfg["M"], cfg["K"], cfg["N"]
        A = torch.from_numpy(cfg["A"]).to(dev)
        B = torch.from_numpy(cfg["B"]).to(dev)
        out = torch.empty(M, N, device=dev)
        need = __import__("ctypes").c_size_t(0)
        from bitwise_spgemm_gb300.capi import call
        call("bsp_spmm_i8_workspace", M, K, __import__("ctypes").byref(need))
        wsp = torch.empty(need.value, dtype=torch.uint8, device=dev)
        step = lambda: ops.spmm_i8(A, B, out=out, workspace=wsp)
        if sampler:
            sampler.start()
        barrier(ws)
        ms = max_over_ranks(ws, _timed(step, steps, warm))
        barrier(ws)
        clocks = sampler.stop() if sampler else None
        planes = ops.bitplanes(A.view(torch.uint8), 8)
        ms_planes = _timed(lambda: ops.bitplanes(A.view(torch.uint8), 8, out=planes), 5, 2)
        ms_prod = _timed(lambda: ops.bitplane_spmm(planes, K, B, out=out), 5, 2)
        nnz = int((cfg["A"] != 0).sum())
        plane_bits = int(np.unpackbits(planes.cpu().numpy().view(np.uint8)).sum())
        # planes along K with bf16 B: one planned bitmap SpMM (tensor cores);
        # the plane-weighted copies of B are stacked inside the timed step
        mat = ops.Int8Matrix(A)
        B16 = B.to(torch.bfloat16)
        Bst = ops.stack_planes_b(B16, K)
        out16 = torch.empty(M, N, device=dev)
        ms_tc = _timed(lambda: mat.matmul(B16, out=out16, B_stacked=Bst), 10, 3)
        tc_info = mat.plan.info()
        mat.close()
        comp = M * K + K * N * 4 + M * N * 4
        sec, rows = _cpu_rows(lambda r: O.bitplane_spmm_f64(cfg["A"][:r], cfg["B"]), M, rows0=16)
        line = dict(base, metric="int8 x dense product GB/s (A int8 + B + C / time)", value=comp / (ms * 1e-3) / 1e9,
                    unit="GB/s", ms_per_step=ms, dtype="f32",
                    config={"workload": cfg["name"], "M": M, "K": K, "N": N, "nnz_A": nnz, "plane_bits": plane_bits,
                            "l2": "inputs (20 MiB) stay in L2"},
                    effective_gflops=2.0 * nnz * N / (ms * 1e-3) / 1e9, bitplanes_ms=ms_planes, product_ms=ms_prod,
                    planes_along_k_bf16={"ms": ms_tc, "speedup_vs_fp32_bitplane": ms / ms_tc,
                                         "occupied_tiles": tc_info["occ_tiles"], "plan_mode": tc_info["mode"]},
                    gather_gbs=plane_bits * N * 4 / (ms_prod * 1e-3) / 1e9,
                    roofline={"bound": "hbm", "achieved": comp / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                              "frac": comp / (ms * 1e-3) / 1e9 / hbm, "traffic": None, "peak_source": hkind},
                    cpu_baseline={"value": comp / sec / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                                  "sample": "oracle bit-plane product (FP64) on the first %d rows, scaled to %d"
                                  % (rows, M)},
                    clocks=clocks)
    else:
        cfg = W.config3()
        M, K = cfg["M"], cfg["K"]
        words = torch.from_numpy(cfg["words"].view(np.int32)).to(dev)
        Mt, Kt = (M + 7) // 8, (K + 7) // 8
        T = Mt * Kt
        bmp = torch.empty(T, dtype=torch.int64, device=dev)
        tr = torch.empty(T, dtype=torch.int32, device=dev)
        tc = torch.empty(T, dtype=torch.int32, device=dev)
        off = torch.empty(T + 1, dtype=torch.int32, device=dev)
        n = torch.empty(1, dtype=torch.int64, device=dev)
        wsp = ops._ws("bsp_tiles8_workspace", M, K, device=dev)
        from bitwise_spgemm_gb300.capi import call
        p = ops._p
        step = lambda: call("bsp_rows_to_tiles8", p(words), M, K, p(bmp), p(tr), p(tc), p(off), p(n), p(wsp),
                            wsp.numel(), ops._stream())
        if sampler:
            sampler.start()
        barrier(ws)
        ms = max_over_ranks(ws, _timed(step, steps, warm))
        barrier(ws)
        clocks = sampler.stop() if sampler else None
        ntiles = int(n.item())
        back = torch.empty_like(words)
        ms_back = _timed(lambda: ops.tiles8_to_rows(bmp[:ntiles], tr[:ntiles], tc[:ntiles], M, K, out=back), 5, 2)
        comp = M * ((K + 31) // 32) * 4 + ntiles * 16 + 4
        t0 = time.perf_counter()
        O.rows_to_tiles8(cfg["words"], M, K)
        cpu_tiles = time.perf_counter() - t0
        c2 = W.config2()
        rp, col = W.bits_to_csr(c2["words"], c2["M"], c2["K"])
        val = np.random.default_rng(14).standard_normal(len(col)).astype(np.float32)
        rp_d, col_d, val_d = (torch.from_numpy(x).to(dev) for x in (rp, col, val))
        ms_csr = _timed(lambda: ops.csr_to_tiled(rp_d, col_d, c2["M"], c2["K"], 512, 2048, values=val_d), 5, 2)
        t0 = time.perf_counter()
        O.csr_to_tiled(rp, col, val, c2["M"], c2["K"], 512, 2048)
        cpu_csr = time.perf_counter() - t0
        line = dict(base, metric="packed rows -> 8x8 bitmap tiles GB/s (words read + tiles written / time)",
                    value=comp / (ms * 1e-3) / 1e9, unit="GB/s", ms_per_step=ms, dtype="u64",
                    config={"workload": "tiles8_" + cfg["name"], "M": M, "K": K, "n_tiles": ntiles,
                            "l2": "32 MiB of words, 8.6 MB of tiles written"},
                    tiles8_to_rows_ms=ms_back,
                    csr_to_tiled={"workload": "csr_" + c2["name"] + "_tiles_512x2048", "nnz": int(len(col)),
                                  "ms": ms_csr, "cpu_ms": cpu_csr * 1e3},
                    roofline={"bound": "hbm", "achieved": comp / (ms * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                              "frac": comp / (ms * 1e-3) / 1e9 / hbm, "traffic": None, "peak_source": hkind},
                    cpu_baseline={"value": comp / cpu_tiles / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                                  "sample": "oracle tile conversion of the full matrix"},
                    clocks=clocks)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "c5":
        run_fwd_bwd(args)
    elif args.config == "c4":
        run_batched(args)
    elif args.config == "c4fb":
        run_batched_fb(args)
    elif args.config == "l2probe":
        run_l2probe(args)
    elif args.config in ("f1", "f2", "f3"):
        run_next(args)
    elif args.config != "c2":
        run_other(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
