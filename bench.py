#!/usr/bin/env python3
"""Headline benchmark: SNICIT-form SDGC inference on one GB300.

Workload (default "sdgc-65536x1920"): N=65536 neurons, L=1920 layers, a batch
of B=60000 seeded binary inputs (per-row density 0.95*Beta(2,8), mean 0.19),
32 nonzeros per weight row at 0.0625, bias -0.45, clamp 32.  One step = one
full inference of the batch through the SNICIT path (plain layers up to the
autotuned threshold, clustering, residue layers, recovery).  Measured beside
it in the same run: the plain per-layer path (SNIG mode) on the same batch,
the end-to-end host API, the dominant kernel alone (roofline), twelve uneven
batches (log-uniform 500..60000 rows) in one launch schedule against one by
one, the 4096 x 480 workload as an extra key, the serving loop, and the CPU
baseline.

Metric: nominal SDGC edges/s = B * 32 * N * L / t (the reference paper's
throughput definition), plus ms per inference.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU recurrence on the host cores.
The reference ships no CPU implementation of the recurrence, so this arm runs
the oracle's FP32 restatement of bf_inference (oracle/sdnn_oracle.c) on a
bounded sample of the same workload with all host threads.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (N, L, B, bias, threshold default)
    "sdgc-1024x120": (1024, 120, 60000, -0.30, 30),
    "sdgc-4096x480": (4096, 480, 60000, -0.35, 30),
    "sdgc-16384x1920": (16384, 1920, 60000, -0.40, 30),
    "sdgc-65536x1920": (65536, 1920, 60000, -0.45, 30),
}
# RadiX-Net-structured nets (radix 2, dense blocks of 16, weights 1/16): extra
# lines only (--extra-workloads)
RADIXNET = {
    "radixnet-1024x120": (1024, 120, 60000, -0.30, 30),
    "radixnet-4096x480": (4096, 480, 60000, -0.35, 30),
    "radixnet-65536x1920": (65536, 1920, 60000, -0.45, 30),
}
SEED = 20260101
NNZ = 32
METRIC = "edges/s & ms/inference, SNICIT vs plain on 1 GB300 (exact categories); p50/p99"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6777.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            with open(self.path) as f:
                for line in f:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) < 9:
                        continue
                    try:
                        sm.append(float(p[1]))
                        mx = max(mx, float(p[2]))
                    except ValueError:
                        continue
                    for n, v in zip(names, p[5:9]):
                        if v.lower().startswith("active"):
                            reasons.add(n)
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_port(N, L, bias, group_rows, row_offset=0):
    """The oracle's FP32 restatement of bf_inference on the host cores over
    consecutive groups of the workload's rows (the weights generated layer by
    layer, untimed); returns (seconds per group, survivors per group, threads)."""
    import numpy as np
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    total = int(sum(group_rows))
    Y = orc.gen_inputs(N, SEED, row_offset, total)
    alive, secs, _ = orc.port_stream(N, L, SEED, bias, Y, group_rows, nnz=NNZ, value=0.0625,
                                     nthreads=threads)
    off = np.concatenate([[0], np.cumsum(group_rows)]).astype(np.int64)
    surv = [int(alive[off[i]:off[i + 1]].sum()) for i in range(len(group_rows))]
    return secs, surv, threads


def cpu_row_seconds(N, L, bias, probe=None):
    """Seconds of host work per input row of the workload, from a probe of a
    few rows (all layers)."""
    threads = os.cpu_count() or 1
    probe = probe or max(2 * threads, 48)
    secs, _, _ = cpu_port(N, L, bias, [probe])
    return max(float(secs[0]), 1e-3) / probe


def cpu_port_rate(N, L, bias, budget_s=12.0):
    """FP32 port on a bounded sample (about budget_s of host work); returns
    (edges/s, rows, seconds, threads)."""
    row_s = cpu_row_seconds(N, L, bias)
    rows = int(min(20000, max(16, budget_s / row_s)))
    secs, _, threads = cpu_port(N, L, bias, [rows])
    return rows * NNZ * N * L / float(secs[0]), rows, float(secs[0]), threads


def run_reference(args):
    import numpy as np
    if args.workload in UNEVEN:
        N, L, bias, nb, lo, hi = UNEVEN[args.workload]
        rng = np.random.default_rng([SEED, 6])
        B = int(np.clip(np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), nb))), lo, hi).sum())
    else:
        N, L, B, bias, _ = WORKLOADS[args.workload]
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # bounded samples: about 2.5 minutes of host work over the timed steps and
    # 12 s over the warm-up ones, whatever K and W are (at most 12 s a step);
    # every step is its own group of consecutive rows of the workload's batch
    row_s = cpu_row_seconds(N, L, bias)
    timed = min(12.0, max(1.0, 150.0 / max(1, args.steps)))
    warm = min(4.0, max(0.5, 12.0 / max(1, args.warmup)))
    sizes = [int(max(16, min(20000, (warm if i < args.warmup else timed) / row_s)))
             for i in range(args.warmup + args.steps)]
    secs, surv, threads = cpu_port(N, L, bias, sizes)
    rates = [n * NNZ * N * L / max(float(t), 1e-9) for n, t in zip(sizes, secs)]
    value = statistics.median(rates[args.warmup:])
    rows = int(np.median(sizes[args.warmup:]))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "edges/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": B * NNZ * N * L / value * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "neurons": N, "layers": L, "batch": B,
                   "nnz_per_row": NNZ, "bias": bias, "mode": "plain recurrence (bf_inference)",
                   "note": "ms_per_step extrapolated from the bounded sample to the whole batch"},
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": f"{rows} consecutive rows of the {B}-row batch per step "
                                   f"({sum(surv[args.warmup:])} survivors over the timed steps), "
                                   f"all {L} layers, median {statistics.median(secs[args.warmup:]):.1f} s "
                                   "of layer arithmetic per step; the reference has no CPU "
                                   "recurrence (src/SDGC/utils/header.h:7-10), so this is the "
                                   "oracle's FP32 restatement of bf_inference"},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def load_weights(eng, args, N, L):
    """Seeded weights, packed on the host and uploaded -- or, with
    --weights-cache DIR, taken from DIR's packed-weight file (written on the
    first run).  Returns where they came from."""
    path = None
    if args.weights_cache:
        os.makedirs(args.weights_cache, exist_ok=True)
        path = os.path.join(args.weights_cache, f"sdgc-{N}x{L}-seed{SEED}.sdnnw")
        if os.path.exists(path):
            eng.load_packed(path)
            eng.finalize()
            return "packed file (mmap)"
    eng.generate_weights(SEED, NNZ, 0.0625)
    eng.finalize()
    if path:
        eng.save_packed(path)
    return "generated + packed"


def uneven_sizes(lo=500, hi=60000, nb=12):
    """Twelve seeded batch sizes, log-uniform in [lo, hi]."""
    import numpy as np
    rng = np.random.default_rng([SEED, 6])
    sizes = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), nb))).astype(np.int64)
    return np.clip(sizes, lo, hi)


def autotune(eng, args, name, d_ptr, rows):
    if args.no_autotune or args.tile:
        return None
    rec = os.path.join(args.record_dir, f"autotune_{name}.jsonl")
    os.makedirs(os.path.dirname(rec), exist_ok=True)
    if os.path.exists(rec):
        os.remove(rec)
    eng.autotune_device(d_ptr, rows, rec)
    return rec


def time_steps(torch, stream, fn, steps):
    """Device time of `steps` calls of fn on `stream` (CUDA events), per step too."""
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per = []
    ev0.record(stream)
    for _ in range(steps):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        fn()
        s1.record(stream)
        per.append((s0, s1))
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), [a.elapsed_time(b) for a, b in per]


def layer_kernel_roofline(torch, sg, eng, d_in, B, N, stream, peak, peak_kind, sm_mhz, args):
    """The dominant kernel alone: layer 1 of the workload (the layer kernel over
    every row of the batch, its inputs the layer-0 outputs) through the
    no-allocation one-layer entry point, timed with CUDA events on the stream
    it is launched on; algorithmic bytes = 8 B per row entry (read + write),
    4 B per row id, 8 B per weight nonzero."""
    import ctypes
    lib = sg.load()
    rows = min(B, 65536)
    y1 = torch.empty((rows, N), dtype=torch.float32, device=d_in.device)
    y2 = torch.empty_like(y1)
    alive = torch.empty(rows, dtype=torch.int32, device=d_in.device)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def call(layer, src, dst):
        rc = lib.sdnn_layer_noalloc(eng._h, layer, ctypes.c_void_p(src.data_ptr()),
                                    ctypes.c_void_p(dst.data_ptr()), rows,
                                    ctypes.c_void_p(alive.data_ptr()), sp)
        assert rc == 0, lib.sdnn_last_error(eng._h)

    call(0, d_in[:rows], y1)
    for _ in range(3):
        call(1, y1, y2)
    n = max(3, min(args.steps, 10))
    # inputs (rows x N x 4 B) are larger than L2 at every workload here
    total_ms, per = time_steps(torch, stream, lambda: call(1, y1, y2), n)
    ms = statistics.median(per)
    nnz = NNZ * N
    algo = 8.0 * N * rows + 4.0 * rows + 8.0 * nnz
    achieved = algo / (ms / 1e3) / 1e9
    del y1, y2, alive
    traffic = None
    prof = os.path.join(ROOT, "profiles", f"layer_kernel_{args.workload}.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    props = torch.cuda.get_device_properties(d_in.device)
    sms = props.multi_processor_count
    smem_gbs = 128.0 * sms * (sm_mhz or 0) * 1e6 / 1e9 if sm_mhz else None
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
            "kernel": f"sdnn::layer_kernel (layer 1 of the workload, {rows} rows)",
            "per": "one launch", "algorithmic_bytes_per_launch": algo, "avg_launch_ms": ms,
            "frac_of_8tbs": achieved / 8000.0,
            "smem_gather_bytes_per_launch": 4.0 * 32 * N * rows,
            "smem_peak_gbs": smem_gbs, "sms": sms, "sm_mhz": sm_mhz}


def run_ours(args):
    import numpy as np
    import torch
    import snicit_gb300 as sg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    N, L, B, bias, t_default = WORKLOADS[args.workload]
    threshold = args.threshold if args.threshold is not None else t_default
    edges = float(B) * NNZ * N * L
    # the twelve uneven batches use the first rows of the same seeded stream,
    # the timed batch the first B of them (each rank its own rows: weak scaling)
    sizes = uneven_sizes() if not args.no_uneven else np.zeros(0, np.int64)
    total_uneven = int(sizes.sum())
    rows_all = max(B, total_uneven)
    d_all = torch.empty((rows_all, N), dtype=torch.float32, device=dev)
    sg.generate_inputs_device(N, SEED, rank * rows_all, rows_all, d_all.data_ptr())
    d_in = d_all[:B]
    d_flags = torch.zeros(B, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    eng = sg.Engine(N, L, mode="SNICIT", threshold=threshold, batch=rows_all, bias=bias,
                    num_centroids=args.centroids, device=local, tile_rows=args.tile,
                    threads=args.threads, merge_start=args.merge_start,
                    merge_every=args.merge_every,
                    device_post_choice=not args.host_post_choice)
    t0 = time.perf_counter()
    weights = load_weights(eng, args, N, L)
    pack_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    record = autotune(eng, args, args.workload, d_in.data_ptr(), args.tune_rows or B)
    tune_s = time.perf_counter() - t0

    # a real (non-default) stream: the engine orders its own stream after it and
    # makes it wait for the engine, so events recorded here bracket the work
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)

    def step():
        eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    flags_ref = d_flags.cpu().numpy().copy()
    if dist:
        dist.barrier()
    with Clocks(local) as clk:
        elapsed_ms, step_ms = time_steps(torch, stream, step, args.steps)
    clocks = clk.summary()
    if dist:
        dist.barrier()
    st = eng.stats()  # stage events of the last step
    flags = d_flags.cpu().numpy()
    assert np.array_equal(flags, flags_ref), "category set changed between steps"
    t = torch.tensor([elapsed_ms], dtype=torch.float64)
    if dist:
        t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    value = world * edges * args.steps / (max_ms / 1e3)
    ms_per_step = max_ms / args.steps

    peak, peak_kind = peaks()
    # the pre-threshold stage as a whole (binary layer 0, layer kernels, merge steps)
    nnz_layer = st["weight_nnz"] / L
    T = st["threshold"]
    pre_bytes = 8.0 * N * st["pre_row_layers"] + 4.0 * st["pre_row_layers"] + 8.0 * nnz_layer * T
    pre_s = st["stage_ms"][0] / 1e3
    pre_stage = {"bytes": pre_bytes, "ms": st["stage_ms"][0],
                 "achieved_gbs": pre_bytes / pre_s / 1e9 if pre_s > 0 else 0.0,
                 "frac": (pre_bytes / pre_s / 1e9) / peak if pre_s > 0 else 0.0,
                 "layers": T, "row_layers": st["pre_row_layers"]}
    roofline = layer_kernel_roofline(torch, sg, eng, d_in, B, N, stream, peak, peak_kind,
                                     clocks.get("sm_mhz"), args)

    # end to end through the public host API: pinned host inputs in, survivor ids out
    host_t = torch.empty((B, N), dtype=torch.float32, pin_memory=True)
    host_t.copy_(d_in)
    host = host_t.numpy()
    n_e2e = max(1, min(args.steps, args.e2e_steps))

    def time_host_calls(fn):
        fn()
        times, n = [], 0
        for _ in range(n_e2e):
            t0 = time.perf_counter()
            _, ids = fn()
            times.append(time.perf_counter() - t0)
            n = len(ids)
        return statistics.median(times), n

    # streamed ingest (the default): the rows copy in pieces and the layers
    # before the first merge run on each piece while the next ones copy
    e2e_s, count = time_host_calls(lambda: eng.infer(host, want_flags=False, want_ids=True))
    pieces = eng.stats()["input_pieces"]
    assert count == int(flags.sum())
    e2e = {"value": world * edges / e2e_s, "unit": "edges/s", "h2d_bytes_per_step": B * N * 4,
           "d2h_bytes_per_step": 4 + 4 * count, "ms_per_step": e2e_s * 1e3,
           "input_pieces": pieces, "api": "sdnn_infer_host (FP32 host rows)"}
    # the same call with one copy of the whole batch before the first layer
    eng.set_input_streaming(-1)
    one_s, count1 = time_host_calls(lambda: eng.infer(host, want_flags=False, want_ids=True))
    eng.set_input_streaming(0)
    assert count1 == count
    e2e_one_copy = {"value": world * edges / one_s, "unit": "edges/s",
                    "h2d_bytes_per_step": B * N * 4, "d2h_bytes_per_step": 4 + 4 * count,
                    "ms_per_step": one_s * 1e3}
    # the same with the inputs as one-bit host rows (the inputs are 0/1): 32x fewer bytes
    bits_t = torch.from_numpy(sg.pack_bits(host)).pin_memory()
    bits = bits_t.numpy()
    e2b_s, count_b = time_host_calls(lambda: eng.infer_bits(bits, want_flags=False, want_ids=True))
    assert count_b == count
    e2e_bits = {"value": world * edges / e2b_s, "unit": "edges/s",
                "h2d_bytes_per_step": int(bits.nbytes), "d2h_bytes_per_step": 4 + 4 * count,
                "ms_per_step": e2b_s * 1e3, "api": "sdnn_infer_host_bits"}
    del host_t, host, bits_t, bits

    # uneven batches in one launch schedule against the same batches one by one
    uneven = None
    if total_uneven:
        offs = np.concatenate([[0], np.cumsum(sizes)])
        u_flags = torch.zeros(total_uneven, dtype=torch.int32, device=dev)
        ptrs = [d_all[int(offs[i])].data_ptr() for i in range(len(sizes))]
        fptrs = [u_flags[int(offs[i]):].data_ptr() for i in range(len(sizes))]
        res = {}
        for name, fn in (("one_schedule", lambda: eng.infer_batches_device(ptrs, sizes, fptrs, stream.cuda_stream)),
                         ("one_by_one", lambda: [eng.infer_device(p, int(n), f, stream.cuda_stream)
                                                 for p, n, f in zip(ptrs, sizes, fptrs)])):
            for _ in range(2):
                fn()
            ms, _ = time_steps(torch, stream, fn, max(1, min(args.steps, 5)))
            res[name] = (ms / max(1, min(args.steps, 5)), u_flags.cpu().numpy().copy())
        u_edges = float(total_uneven) * NNZ * N * L
        uneven = {"batches": sizes.tolist(), "rows": total_uneven,
                  "one_schedule_ms": res["one_schedule"][0], "one_by_one_ms": res["one_by_one"][0],
                  "edges_per_s": u_edges / (res["one_schedule"][0] / 1e3),
                  "speedup_vs_one_by_one": res["one_by_one"][0] / res["one_schedule"][0],
                  "category_sets_equal": bool(np.array_equal(res["one_schedule"][1],
                                                             res["one_by_one"][1])),
                  "survivors": int(res["one_schedule"][1].sum())}
        del u_flags

    # plain per-layer path (SNIG mode) on the same batch and the same resident weights
    eng.set_mode("SNIG", L)
    plain_flags = torch.zeros(B, dtype=torch.int32, device=dev)
    eng.infer_device(d_in.data_ptr(), B, plain_flags.data_ptr(), stream.cuda_stream)
    psteps = max(1, min(args.steps, 3))
    p_ms, _ = time_steps(torch, stream, lambda: eng.infer_device(
        d_in.data_ptr(), B, plain_flags.data_ptr(), stream.cuda_stream), psteps)
    plain_ms = p_ms / psteps
    pst = eng.stats()
    plain_exact = bool(np.array_equal(plain_flags.cpu().numpy(), flags))
    launches = st["launches"] * args.steps
    eng.close()
    del d_all, d_in, plain_flags
    torch.cuda.empty_cache()

    extra = {}
    if rank == 0 and not args.no_extra:
        for wl in args.extra_workloads.split(","):
            if wl and wl != args.workload:
                extra[wl] = run_extra(args, sg, torch, wl, local)
        if not args.no_residue:
            extra["residue_stage"] = run_residue(args, sg, torch, local)

    cpu = None
    if rank == 0 and not args.no_cpu:
        r, rows, secs, threads = cpu_port_rate(N, L, bias, args.cpu_seconds)
        cpu = {"value": r, "unit": "edges/s", "cores": threads, "kind": "port",
               "sample": f"first {rows} rows of the batch, all {L} layers, {secs:.1f} s of "
                         "layer arithmetic (FP32 restatement of bf_inference)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": args.workload, "neurons": N, "layers": L, "batch": B,
                       "nnz_per_row": NNZ, "bias": bias, "mode": "SNICIT",
                       "threshold": st["threshold"], "centroids_kept": st["centroids"],
                       "centroid_candidates": st["centroid_candidates"],
                       "merge_start": st["merge_start"], "merge_every": st["merge_every"],
                       "post_kernel": st["post_kernel"],
                       "tile_rows": st["tile_rows"], "threads": st["threads"],
                       "l2": "inputs (B*N*4 bytes) larger than L2",
                       "parallelism": f"replicas x{world} (independent batches)"},
            "p50_ms": statistics.median(step_ms),
            "p99_ms": sorted(step_ms)[min(len(step_ms) - 1, int(0.99 * len(step_ms)))],
            "survivors": int(flags.sum()),
            "stage_ms": st["stage_ms"],
            "pack_s": pack_s, "weights": weights, "autotune_s": tune_s,
            "autotune_record": os.path.relpath(record, ROOT) if record else None,
            "plain": {"ms_per_inference": plain_ms, "edges_per_s": edges / (plain_ms / 1e3),
                      "category_set_equal": plain_exact, "row_layers": pst["row_layers"]},
            "speedup_vs_plain": plain_ms / ms_per_step,
            "roofline": roofline, "pre_stage": pre_stage, "cpu_baseline": cpu, "e2e": e2e,
            "e2e_one_copy": e2e_one_copy, "e2e_bit_inputs": e2e_bits,
            "uneven": uneven,
            "gpu_launches": launches,
            "clocks": clocks,
        }
        line.update(extra)
        if not args.no_serve:
            line["serving"] = run_serving(args, sg, local)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_residue(args, sg, torch, local, workload="sdgc-4096x480", threshold=6):
    """A workload where residue rows persist past the threshold: the 4096 x 480
    net clustered at layer 6 (rows not yet saturated) without merging, with
    sparse residue lists and with dense residue rows only.  Reports the
    post-threshold stage: time, residue row-layers (dense + sparse) and the
    algorithmic bytes per second of the residue update."""
    import numpy as np
    N, L, B, bias, _ = WORKLOADS[workload]
    dev = f"cuda:{local}"
    d_in = torch.empty((B, N), dtype=torch.float32, device=dev)
    sg.generate_inputs_device(N, SEED, 0, B, d_in.data_ptr())
    d_flags = torch.zeros(B, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    out = {"workload": workload, "threshold": threshold, "merge": False}
    flags = {}
    for sparse in (True, False):
        with sg.Engine(N, L, mode="SNICIT", threshold=threshold, batch=B, bias=bias,
                       num_centroids=args.centroids, device=local, merge=False,
                       sparse_residue=sparse) as eng:
            eng.generate_weights(SEED, NNZ, 0.0625)
            eng.finalize()
            fn = lambda: eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr(), stream.cuda_stream)
            for _ in range(2):
                fn()
            n = max(3, min(args.steps, 10))
            ms, _ = time_steps(torch, stream, fn, n)
            st = eng.stats()
            flags[sparse] = d_flags.cpu().numpy().copy()
            rl = eng.layer_rows()
        post_ms = st["stage_ms"][2]
        res_layers = int(st["post_row_layers"] - st["centroids"] * (L - threshold))
        # per residue row-layer: read + write the row (8 N B) and the centroid
        # pre-activations (4 N B) for dense rows; sparse rows count the same
        # here (upper bound of what a dense update moves)
        algo = 12.0 * N * res_layers + 8.0 * NNZ * N * (L - threshold)
        out["sparse" if sparse else "dense"] = {
            "ms_per_inference": ms / n, "post_stage_ms": post_ms,
            "residue_rows_at_threshold": st["residue_rows"],
            "sparse_rows_at_threshold": st["sparse_residue_rows"],
            "residue_row_layers": res_layers, "sparse_row_layers": st["sparse_row_layers"],
            "post_layers_with_residues": int(sum(1 for l in range(threshold, L)
                                                 if rl[l] > st["centroids"])),
            "post_dense_equivalent_gbs": algo / (post_ms / 1e3) / 1e9 if post_ms > 0 else None,
            "survivors": int(flags[sparse].sum())}
    out["category_sets_equal"] = bool(np.array_equal(flags[True], flags[False]))
    out["post_speedup_sparse_vs_dense"] = (out["dense"]["post_stage_ms"] /
                                           max(out["sparse"]["post_stage_ms"], 1e-9))
    del d_in, d_flags
    torch.cuda.empty_cache()
    return out


def run_density(args):
    """Live rows and the nonzero density of the live rows' activations after
    each of the first layers (the inputs of the next layer), stepping one
    engine's layers with the one-layer entry point on seeded rows -- the
    figures that decide whether skipping zero inputs could beat the gather."""
    import ctypes
    import torch
    import snicit_gb300 as sg
    N, L, B, bias, _ = WORKLOADS[args.workload]
    rows = min(args.density_rows, 65536)
    K = min(args.density_layers, L)
    lib = sg.load()
    x = torch.empty((rows, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, SEED, 0, rows, x.data_ptr())
    y = torch.empty_like(x)
    alive = torch.empty(rows, dtype=torch.int32, device="cuda")
    out = {"workload": args.workload, "rows": rows, "layers": []}
    with sg.Engine(N, K, mode="SNIG", batch=rows, bias=bias) as eng:
        eng.generate_weights(SEED, NNZ, 0.0625)
        eng.finalize()
        live_in = rows
        out["input_density"] = float((x > 0).float().mean())
        for l in range(K):
            rc = lib.sdnn_layer_noalloc(eng._h, l, ctypes.c_void_p(x.data_ptr()),
                                        ctypes.c_void_p(y.data_ptr()), rows,
                                        ctypes.c_void_p(alive.data_ptr()), None)
            assert rc == 0, lib.sdnn_last_error(eng._h)
            torch.cuda.synchronize()
            m = alive > 0
            live = int(m.sum())
            yl = y[m]
            dens = float((yl > 0).float().mean()) if live else 0.0
            sat = float((yl >= 32.0).float().mean()) if live else 0.0
            out["layers"].append({"layer": l, "rows_in": live_in, "rows_out": live,
                                  "out_density": dens, "saturated": sat})
            live_in = live
            x, y = y, x
    print(json.dumps({"density": out}), flush=True)


def run_extra(args, sg, torch, workload, local):
    """Another SDGC workload on the same GPU, reported as an extra key: SNICIT
    (autotuned) and the plain path, device-resident inputs."""
    import numpy as np
    N, L, B, bias, t_default = WORKLOADS[workload] if workload in WORKLOADS else RADIXNET[workload]
    dev = f"cuda:{local}"
    d_in = torch.empty((B, N), dtype=torch.float32, device=dev)
    sg.generate_inputs_device(N, SEED, 0, B, d_in.data_ptr())
    d_flags = torch.zeros(B, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    with sg.Engine(N, L, mode="SNICIT", threshold=t_default, batch=B, bias=bias,
                   num_centroids=args.centroids, device=local) as eng:
        if workload in RADIXNET:
            eng.generate_radixnet(16, 0.0625)
        else:
            eng.generate_weights(SEED, NNZ, 0.0625)
        eng.finalize()
        autotune(eng, args, workload, d_in.data_ptr(), B)
        fn = lambda: eng.infer_device(d_in.data_ptr(), B, d_flags.data_ptr(), stream.cuda_stream)
        for _ in range(args.warmup):
            fn()
        ms, per = time_steps(torch, stream, fn, args.steps)
        st = eng.stats()
        flags = d_flags.cpu().numpy().copy()
        eng.set_mode("SNIG", L)
        fn()
        pms, _ = time_steps(torch, stream, fn, 3)
        plain = d_flags.cpu().numpy()
    edges = float(B) * NNZ * N * L
    del d_in, d_flags
    torch.cuda.empty_cache()
    return {"workload": workload, "ms_per_inference": ms / args.steps,
            "edges_per_s": edges / (ms / args.steps / 1e3), "p50_ms": statistics.median(per),
            "plain_ms": pms / 3, "speedup_vs_plain": (pms / 3) / (ms / args.steps),
            "category_set_equal": bool(np.array_equal(flags, plain)),
            "survivors": int(flags.sum()), "stage_ms": st["stage_ms"],
            "threshold": st["threshold"], "tile_rows": st["tile_rows"],
            "threads": st["threads"], "merge_start": st["merge_start"]}


UNEVEN = {
    # name: (N, L, bias, batches, smallest, largest)
    "uneven-65536x1920": (65536, 1920, -0.45, 12, 500, 60000),
    "uneven-4096x480": (4096, 480, -0.35, 12, 500, 60000),
}


def run_uneven(args):
    """Twelve seeded batches of log-uniform sizes run as one launch schedule
    (sdnn_infer_batches_device) against the same batches one by one."""
    import numpy as np
    import torch
    import snicit_gb300 as sg
    torch.cuda.set_device(0)
    N, L, bias, nb, lo, hi = UNEVEN[args.workload]
    rng = np.random.default_rng([SEED, 6])
    sizes = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), nb))).astype(np.int64)
    sizes = np.clip(sizes, lo, hi)
    total = int(sizes.sum())
    offs = np.concatenate([[0], np.cumsum(sizes)])
    d_in = torch.empty((total, N), dtype=torch.float32, device="cuda")
    sg.generate_inputs_device(N, SEED, 0, total, d_in.data_ptr())
    d_flags = torch.zeros(total, dtype=torch.int32, device="cuda")
    ptrs = [d_in[offs[i]].data_ptr() for i in range(nb)]
    fptrs = [d_flags[offs[i]:].data_ptr() for i in range(nb)]
    eng = sg.Engine(N, L, mode="SNICIT", threshold=30, batch=total, bias=bias,
                    num_centroids=args.centroids, tile_rows=args.tile, threads=args.threads)
    eng.generate_weights(SEED, NNZ, 0.0625)
    t0 = time.perf_counter()
    eng.finalize()
    pack_s = time.perf_counter() - t0
    if not args.no_autotune and not args.tile:
        rec = os.path.join(args.record_dir, f"autotune_{args.workload}.jsonl")
        os.makedirs(os.path.dirname(rec), exist_ok=True)
        if os.path.exists(rec):
            os.remove(rec)
        eng.autotune_device(ptrs[int(np.argmax(sizes))], int(sizes.max()), rec)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def together():
        eng.infer_batches_device(ptrs, sizes, fptrs, stream.cuda_stream)

    def one_by_one():
        for p, n, f in zip(ptrs, sizes, fptrs):
            eng.infer_device(p, int(n), f, stream.cuda_stream)

    res = {}
    for name, fn in (("one_schedule", together), ("one_by_one", one_by_one)):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(0) as clk:
            ev0.record(stream)
            for _ in range(args.steps):
                fn()
            ev1.record(stream)
            torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        res[name] = {"ms": ms, "flags": d_flags.cpu().numpy().copy(), "clocks": clk.summary(),
                     "stats": eng.stats()}
    same = bool(np.array_equal(res["one_schedule"]["flags"], res["one_by_one"]["flags"]))
    edges = float(total) * NNZ * N * L
    st = res["one_schedule"]["stats"]
    line = {
        "metric": METRIC, "value": edges / (res["one_schedule"]["ms"] / 1e3), "unit": "edges/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["one_schedule"]["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "neurons": N, "layers": L, "batch_sizes": sizes.tolist(),
                   "rows": total, "bias": bias, "mode": "SNICIT", "threshold": st["threshold"],
                   "tile_rows": st["tile_rows"], "threads": st["threads"],
                   "merge_start": st["merge_start"]},
        "one_by_one": {"ms_per_step": res["one_by_one"]["ms"],
                       "edges_per_s": edges / (res["one_by_one"]["ms"] / 1e3)},
        "speedup_vs_one_by_one": res["one_by_one"]["ms"] / res["one_schedule"]["ms"],
        "category_sets_equal": same, "survivors": int(res["one_schedule"]["flags"].sum()),
        "stage_ms": st["stage_ms"], "pack_s": pack_s,
        "gpu_launches": st["launches"] * args.steps,
        "clocks": res["one_schedule"]["clocks"],
    }
    print(json.dumps(line), flush=True)
    eng.close()


def _percentile(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(q * len(xs)))] if xs else None


def serve_stream(sg, eng, head_w, head_b, pool, arrivals, sizes, offsets, **server_kw):
    """Replays a request stream against a Server; returns (latencies s, rows, wall s, stats)."""
    with sg.Server(eng, head_w, head_b, **server_kw) as sv:
        sv.wait(sv.submit(pool[:64]))  # first pass: graph capture, not part of the stream
        ids = [None] * len(sizes)

        def submitter():
            t0 = time.perf_counter()
            for i, (a, n, o) in enumerate(zip(arrivals, sizes, offsets)):
                d = t0 + a - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                ids[i] = sv.submit(pool[o:o + n])

        t_start = time.perf_counter()
        th = threading.Thread(target=submitter)
        th.start()
        lat = []
        for i in range(len(sizes)):
            while ids[i] is None:
                time.sleep(1e-4)
            lat.append(sv.wait(ids[i]).latency_s)
        wall = time.perf_counter() - t_start
        th.join()
        st = sv.stats()
    return lat, int(sum(sizes)), wall, st


def serving_setup(args, sg, local=0):
    """The serving workload: the sparse MLP, the request stream, the input
    pool and one engine per mode (the SNICIT one autotuned)."""
    import numpy as np
    N, L = 1024, 120
    layers, hw, hb = sg.sparse_mlp(SEED, N=N, L=L)
    arrivals, sizes = sg.request_stream(SEED, args.serve_requests, rate=args.serve_rate)
    pool = sg.mlp_inputs(SEED, 0, 16384, N)
    rng = np.random.default_rng([SEED, 5])
    offsets = [int(rng.integers(0, len(pool) - n + 1)) for n in sizes]
    engines = {}
    for mode in ("SNICIT", "SNIG"):
        e = sg.Engine(N, L, mode=mode, threshold=30, batch=4096, bias=-0.05, num_centroids=50,
                      device=local)
        for l, (ro, c, v) in enumerate(layers):
            e.set_layer_csr(l, ro, c, v)
        engines[mode] = e
    # the SNICIT engine's settings come from the autotuner on a sample pass of
    # the pool (threshold, centroids, sparse or dense residues, merging -- or
    # no clustering at all); the server's slots take them over
    rec = os.path.join(args.record_dir, "autotune_serve-mlp-1024x120.jsonl")
    os.makedirs(os.path.dirname(rec), exist_ok=True)
    if os.path.exists(rec):
        os.remove(rec)
    tuned = engines["SNICIT"].autotune(pool[:4096], rec)
    return dict(N=N, L=L, hw=hw, hb=hb, arrivals=arrivals, sizes=sizes, pool=pool,
                offsets=offsets, engines=engines, tuned=tuned)


def run_serve_sweep(args, sg):
    """Slots x rows-per-slot grid of the continuous-batching server on the
    serving workload; one JSON line per point."""
    w = serving_setup(args, sg)
    for mode in ("SNIG", "SNICIT"):
        for slots in (1, 2, 3, 4, 6):
            for max_rows in (16384, 8192, 4096):
                lat, rows, wall, st = serve_stream(sg, w["engines"][mode], w["hw"], w["hb"],
                                                   w["pool"], w["arrivals"], w["sizes"],
                                                   w["offsets"], slots=slots, max_rows=max_rows)
                print(json.dumps({"mode": mode, "slots": slots, "max_rows": max_rows,
                                  "p50_ms": _percentile(lat, 0.5) * 1e3,
                                  "p99_ms": _percentile(lat, 0.99) * 1e3,
                                  "samples_per_s": rows / wall, "passes": st["passes"]}),
                      flush=True)
    for e in w["engines"].values():
        e.close()


def run_serving(args, sg, local=0):
    """Serving loop on the sparse MLP (1024 inputs, 120 layers of width 1024 at
    3% density, N(0, 0.3^2) weights, bias -0.05, clamp 32, dense 1024x10 head):
    a seeded Poisson stream of requests (sizes log-uniform in [1, 4096]) at
    --serve-rate req/s, replayed in real time against the continuous-batching
    server (SNICIT mode, clustering across co-resident requests, and SNIG
    mode), against the per-request path (one request per pass, SNIG), and at
    saturation (all requests queued at once)."""
    import numpy as np
    w = serving_setup(args, sg, local)
    N, L, hw, hb, pool = w["N"], w["L"], w["hw"], w["hb"], w["pool"]
    arrivals, sizes, offsets, engines, tuned = (w["arrivals"], w["sizes"], w["offsets"],
                                                w["engines"], w["tuned"])
    out = {"workload": f"serve-mlp-{N}x{L}", "requests": len(sizes), "rate_req_s": args.serve_rate,
           "rows": int(sizes.sum()), "mean_rows": float(sizes.mean()),
           "arrival_span_s": float(arrivals[-1])}
    out["snicit_settings"] = {k: tuned[k] for k in ("threshold", "centroid_candidates",
                                                      "merge_start", "tile_rows", "threads")}
    # continuous batching: four slots of at most 4096 rows each, so a request
    # that arrives during a pass waits for a short pass, not a 16384-row one;
    # saturation: two slots of 16384 rows (throughput)
    live = dict(slots=4, max_rows=4096)
    bulk = dict(slots=2, max_rows=16384)
    arms = [("continuous_snicit", "SNICIT", live, arrivals),
            ("continuous_plain", "SNIG", live, arrivals),
            ("per_request_plain", "SNIG", dict(slots=1, max_requests_per_pass=1, max_rows=16384),
             arrivals),
            ("saturation_snicit", "SNICIT", bulk, np.zeros_like(arrivals)),
            ("saturation_plain", "SNIG", bulk, np.zeros_like(arrivals))]
    out["continuous_server"] = live
    for name, mode, kw, arr in arms:
        lat, rows, wall, st = serve_stream(sg, engines[mode], hw, hb, pool, arr, sizes, offsets,
                                           **kw)
        out[name] = {"samples_per_s": rows / wall, "p50_ms": _percentile(lat, 0.5) * 1e3,
                     "p99_ms": _percentile(lat, 0.99) * 1e3, "passes": st["passes"],
                     "max_rows_in_pass": st["max_rows_in_pass"], "wall_s": wall}
    for e in engines.values():
        e.close()
    return out


CASES = {
    # name: (N, L, rows, mode, threshold) -- small fixed cases for ncu captures
    "plain-n4096": (4096, 6, 8192, "SNIG", 6),
    "chain-n4096": (4096, 60, 4096, "SNICIT", 30),
    "plain-n65536": (65536, 3, 2048, "SNIG", 3),
    "plain-n4096-30k": (4096, 3, 30000, "SNIG", 3),
    "chain-n65536": (65536, 40, 2048, "SNICIT", 30),
    "plain-n65536-4k": (65536, 3, 4096, "SNIG", 3),
    "plain-n16384": (16384, 3, 16384, "SNIG", 3),
    "residue-n16384": (16384, 24, 4096, "SNICIT", 6),
}


def run_case(args):
    """One small engine run (two inferences) for profiling; prints its stats."""
    import snicit_gb300 as sg
    N, L, B, mode, t = CASES[args.case]
    Y0 = sg.generate_inputs(N, SEED, 0, B)
    eng = sg.Engine(N, L, mode=mode, threshold=t, batch=B, bias=sg.load().sdnn_reference_bias(N),
                    num_centroids=args.centroids, tile_rows=args.tile, threads=args.threads,
                    merge_start=args.merge_start, merge_every=args.merge_every,
                    merge=not args.case.startswith("residue"),
                    # ncu cannot profile kernels inside a graph with a conditional
                    # node: the cases let the host choose the post path
                    device_post_choice=False,
                    sparse_residue=not args.dense_residue)
    eng.generate_weights(SEED, NNZ, 0.0625)
    for _ in range(2):
        eng.infer(Y0)
    print(json.dumps({"case": args.case, "stats": eng.stats()}), flush=True)
    eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sdgc-65536x1920", choices=sorted(WORKLOADS) + sorted(UNEVEN))
    ap.add_argument("--threshold", type=int, default=None)
    ap.add_argument("--centroids", type=int, default=50)
    ap.add_argument("--tune-rows", type=int, default=0, help="rows used by the autotuner (0 = all)")
    ap.add_argument("--tile", type=int, default=0, help="fix the layer-kernel tile rows (skips autotune)")
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--merge-start", type=int, default=0,
                    help="first layer after which identical rows merge (0 = default/autotuned)")
    ap.add_argument("--merge-every", type=int, default=0)
    ap.add_argument("--record-dir", default=os.path.join(ROOT, "records"),
                    help="where the autotuner's JSON-lines record of its sweep goes")
    ap.add_argument("--weights-cache", default=None,
                    help="directory of packed-weight files (written on the first run)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-uneven", action="store_true",
                    help="skip the twelve uneven batches (one schedule vs one by one)")
    ap.add_argument("--no-extra", action="store_true", help="skip the extra workloads")
    ap.add_argument("--no-residue", action="store_true",
                    help="skip the residue-stage measurement (4096 x 480 clustered at layer 6)")
    ap.add_argument("--residue-only", action="store_true",
                    help="only the residue-stage measurement")
    ap.add_argument("--host-post-choice", action="store_true",
                    help="the host picks the post-threshold path (phase graphs without a "
                         "conditional node, whose kernels ncu can profile)")
    ap.add_argument("--dense-residue", action="store_true",
                    help="cases: every residue row stays dense (no sparse lists)")
    ap.add_argument("--density", action="store_true",
                    help="live rows and activation density per layer of --workload")
    ap.add_argument("--density-rows", type=int, default=8192)
    ap.add_argument("--density-layers", type=int, default=12)
    ap.add_argument("--extra-workloads", default="sdgc-4096x480,radixnet-4096x480",
                    help="comma-separated workloads reported as extra keys")
    ap.add_argument("--e2e-steps", type=int, default=5,
                    help="host-API calls timed per end-to-end form (median)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serve-only", action="store_true", help="only the serving-loop measurement")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-sweep", action="store_true",
                    help="slots x rows-per-slot grid of the serving loop, one JSON line each")
    ap.add_argument("--case", default=None, choices=sorted(CASES),
                    help="run a small fixed case (used for ncu captures) instead of the bench")
    args = ap.parse_args()
    if args.case:
        run_case(args)
    elif args.density:
        run_density(args)
    elif args.residue_only:
        import torch
        import snicit_gb300 as sg
        print(json.dumps({"residue_stage": run_residue(args, sg, torch, 0)}), flush=True)
    elif args.serve_sweep:
        import snicit_gb300 as sg
        run_serve_sweep(args, sg)
    elif args.serve_only:
        import snicit_gb300 as sg
        print(json.dumps({"serving": run_serving(args, sg)}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload in UNEVEN:
        run_uneven(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
