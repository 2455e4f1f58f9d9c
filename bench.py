"""Benchmark of the grid2grid transform path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
                    [--impl ours|reference]

Workload (default): random_grid_f32_16384 -- float 16384 x 16384 redistributed
between two arbitrary grid-like layouts over 16 virtual ranks (random split
points with extents U[1, 2048], random owners, every block separately
allocated with a padded stride), seeded random bit patterns.

A step is one transform of that matrix. `value` is redistributed GB/s
(m*n*sizeof(T) per step / time) with the layouts resident in HBM and the plan
cached: the device-timed gather-scatter. `e2e` is the same metric through the
host-buffer call a CPU caller makes: host-to-device copy of the initial
layout from pinned memory, plan + transform (the reference's transform also
re-plans every call), device-to-host copy of the final layout.

`--impl reference` times the reference algorithm on the host cores (the
reference library itself where it was built for this host, else the
project's CPU restatement of it) on the same workload and prints the same
line with "impl": "reference".

Multi-GPU: `--gpus N` runs an independent replica per rank, `value` is the
sum over ranks, timing is max over ranks ("scaling": "weak"). The sharded
transform (virtual ranks spread over GPUs, grid2grid_gb300/exchange.py) is
timed as `sharded_loopback`: two shards on one GPU, pack, buffer exchange
and unpack.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "redistributed GB/s"
UNIT = "GB/s"


# GB300 HBM3e datasheet bandwidth (the "about 8 TB/s" figure), reported
# beside the measured copy peak that the fractions use.
NOMINAL_HBM_GBS = 7900.0


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_traffic(kernel: str, workload: str):
    """dram bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(p):
        return None
    m = re.search(r"dram_bytes_per_launch\s*=\s*([0-9]+)", open(p).read())
    return int(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled in the background."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, period_ms: int = 20):
        self.index = index
        self.period = period_ms
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", f"-lms={self.period}"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t0 = time.time()
        while not self.samples and time.time() - t0 < 3.0:
            time.sleep(0.01)
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        win = [p for (t, p) in self.samples if t0 - 0.05 <= t <= t1 + 0.05]
        if not win:
            win = [p for (_, p) in self.samples[-3:]]
        if not win:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"],
                    "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(p[1]) for p in win if num(p[1]) is not None]
        mx = [num(p[2]) for p in win if num(p[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for p in win for k in range(4)
                          if p[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(win)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _allreduce_max(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(bytes_per_step: int, ms_per_step_max: float, world_size: int) -> float:
    """Whole-job GB/s of independent replicas: every rank moves bytes_per_step
    per step; the job's step time is the slowest rank's."""
    return bytes_per_step * world_size / (ms_per_step_max * 1e-3) / 1e9


def _cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu_reference(w, reps: int, threads: int, host_arenas=None):
    """Times the reference algorithm on the host: the reference library when it
    was built for this host (oracle/_ref), else the oracle port. Returns
    (seconds per transform list, kind, sample description)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from grid2grid_gb300 import workloads as W
    if host_arenas is None:
        ia, fa = W.fill_arenas(w)
    else:
        ia, fa = host_arenas
    kind = "port"
    use_ref = False
    if oracle.ref_available() and len({L.dtype for L in w.inits}) == 1:
        try:
            oracle.ref()
            use_ref = True
            kind = "reference"
        except OSError:
            use_ref = False
    if not use_ref:
        oracle.build_port()
    times = []
    ops = None if w.ops is None else list(w.ops)
    from grid2grid_gb300 import capi
    for r in range(reps + 1):
        fcopy = [a.copy() for a in fa]
        t0 = time.perf_counter()
        if use_ref:
            oracle.ref_transform(w.inits, w.finals, ia, fcopy,
                                 None if ops is None else [capi.make_op(*o) for o in ops],
                                 oracle.MODE_SINGLE_SCALED if ops else oracle.MODE_SINGLE)
        else:
            oracle.port_transform(w.inits, w.finals, ia, fcopy, ops, threads=threads)
        dt = time.perf_counter() - t0
        if r > 0:  # first run warms page tables and caches
            times.append(dt)
    ranks = max(L.n_ranks for L in w.inits + w.finals)
    sample = (f"{w.name}: full transform x{reps} after 1 warm-up; "
              f"{ranks} ranks as {'thread-MPI ranks' if use_ref else 'threads'}"
              f" on {threads} host threads")
    return times, kind, sample


def run_reference_arm(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from grid2grid_gb300 import workloads as W
    w = W.BY_NAME[args.workload]()
    threads = _cpu_threads()
    reps = max(1, args.steps)
    times, kind, sample = time_cpu_reference(w, reps + max(0, args.warmup - 1), threads)
    times = times[-reps:]
    sec = statistics.median(times)
    value = w.bytes_moved / sec / 1e9
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": reps, "warmup": args.warmup,
        "ms_per_step": round(sec * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": _dtype_name(w), "data": "synthetic (seeded)",
        "config": _config(w, args),
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                         "kind": kind, "sample": sample},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _dtype_name(w):
    from grid2grid_gb300 import capi
    names = sorted({capi.DTYPE_NAME[L.dtype] for L in w.inits})
    short = {"float32": "f32", "float64": "f64", "complex64": "c64", "complex128": "c128"}
    return "+".join(short[n] for n in names)


def _config(w, args):
    c = {"workload": w.name}
    c.update(w.meta)
    c["bytes_per_step"] = w.bytes_moved
    c["l2"] = "inputs larger than L2 (no flush)" if w.bytes_moved >= 512 * 2**20 else \
        "L2 flushed between steps (512 MiB write, then 256 MiB read of another buffer)"
    c["parallelism"] = f"replicas x{args.gpus}"
    if getattr(args, "alpha_beta", None) is not None:
        c["alpha_beta"] = list(args.alpha_beta)
    return c


def run_ours(args):
    import torch
    from grid2grid_gb300 import capi
    from grid2grid_gb300 import workloads as W
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    # room in the one-shot plan cache for the 256 transforms of the batch
    os.environ.setdefault("G2G_PLAN_CACHE_ENTRIES", "512")
    lib = capi.load()
    w = W.BY_NAME[args.workload]()
    dev = torch.device("cuda", local)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    dev_i = [torch.randint(0, 256, (L.arena_bytes,), dtype=torch.uint8, device=dev,
                           generator=gen) for L in w.inits]
    dev_f = [torch.randint(0, 256, (L.arena_bytes,), dtype=torch.uint8, device=dev,
                           generator=gen) for L in w.finals]
    keep = []

    def descs(layouts, tensors):
        arr = (capi.LayoutDesc * len(layouts))()
        for k, (L, t) in enumerate(zip(layouts, tensors)):
            d, kk = L.desc(t.data_ptr())
            arr[k] = d
            keep.append(kk)
        return arr

    n = len(w.inits)
    dI, dF = descs(w.inits, dev_i), descs(w.finals, dev_f)
    dts = (C.c_int * n)(*w.dtypes())
    ops = None
    if args.alpha_beta is not None: # the workload's op letters, scaled
        a, b = args.alpha_beta
        ops = (capi.Op * n)(*[capi.make_op(w.ops[k][0] if w.ops else "N", a, b)
                              for k in range(n)])
    elif w.ops is not None:
        ops = (capi.Op * n)(*[capi.make_op(*o) for o in w.ops])
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)
    plan = C.c_void_p()
    t_plan0 = time.perf_counter()
    capi.check(lib.g2g_plan_create_batch(n, dI, dF, dts, ops, sp, C.byref(plan)))
    plan_ms = (time.perf_counter() - t_plan0) * 1e3
    if args.tuning:  # explicit kernel knobs, e.g. to profile one variant
        t = capi.Tuning()
        for kv in args.tuning.split(","):
            k, v = kv.split("=")
            setattr(t, k.strip(), int(v))
        capi.check(lib.g2g_plan_set_tuning(plan, C.byref(t)))
    tuned = None
    default_ms = None
    # the autotuner times repeated executions back to back, so for a working
    # set that fits in L2 it would rank L2 hits: those plans keep the default
    if args.autotune and not args.tuning and w.bytes_moved >= 512 * 2**20:
        # the library's autotuner picks the knobs of the cached plan before the
        # timed region (the default tuning's time is reported beside)
        default_ms = _plan_kernel_ms(plan, sp, stream, 10, w.bytes_moved < 512 * 2**20, dev)
        t = capi.Tuning()
        capi.check(lib.g2g_plan_autotune(plan, sp, 3, C.byref(t)))
        tuned = {k: getattr(t, k) for k in ("tile_bytes", "tile_dim", "ctas_per_sm",
                                            "threads", "unroll", "stages", "ring",
                                            "tile_run", "l2_prefetch", "tensor_boxes")}
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    # warm-up
    for _ in range(args.warmup):
        capi.check(lib.g2g_plan_execute(plan, sp))
    stream.synchronize()
    sampler = ClockSampler(local).start() if rank == 0 else None
    # timed region: one launch per step, events around each launch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    _barrier(ws)
    torch.cuda.synchronize()
    t_wall0 = time.time()
    # workloads that fit in L2 get it flushed before every step, outside the
    # per-step events: a 512 MiB write, then a 256 MiB read of another buffer
    # so that the write's dirty lines are written back before the step
    # starts instead of during it
    flush = flush_rd = None
    if w.bytes_moved < 512 * 2**20:
        flush = torch.empty(512 * 2**20, dtype=torch.uint8, device=dev)
        flush_rd = torch.ones(32 * 2**20, dtype=torch.int64, device=dev)
    start_all = torch.cuda.Event(enable_timing=True)
    end_all = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start_all.record(stream)
        for k in range(args.steps):
            if flush is not None:
                flush.zero_()
                flush_rd.sum()
            ev[k][0].record(stream)
            capi.check(lib.g2g_plan_execute(plan, sp))
            ev[k][1].record(stream)
        end_all.record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    _barrier(ws)
    t_wall1 = time.time()
    launch_ms = [a.elapsed_time(b) for a, b in ev]
    # per step: the transform itself (the flush, when there is one, is not
    # part of the step)
    total_ms = sum(launch_ms) if flush is not None else start_all.elapsed_time(end_all)
    total_ms = _allreduce_max(total_ms, ws)
    ms_per_step = total_ms / args.steps
    kernel_ms = statistics.mean(launch_ms)
    clocks = None
    if sampler is not None:
        time.sleep(0.06)
        sampler.stop()
        clocks = sampler.summary(t_wall0, t_wall1)
    bytes_step = info.bytes_moved
    value = replica_value(bytes_step, ms_per_step, ws)
    peak, peak_kind = _peaks()
    achieved = info.bytes_min_traffic / (kernel_ms * 1e-3) / 1e9
    # the scaled kernel's capture is its own summary (profiles/*_scaled.md)
    traffic = _profile_traffic("g2g_scatter", w.name + ("_scaled" if args.alpha_beta else ""))
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": info.bytes_min_traffic,
                "kernel_ms": round(kernel_ms, 5),
                "nominal_peak": NOMINAL_HBM_GBS,
                "frac_of_nominal": round(achieved / NOMINAL_HBM_GBS, 4)}

    # e2e: host buffers through the host-layout call, copies inside the timing
    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(lib, w, dev_i, dev_f, args.e2e_steps, stream, ws)
    capi.check(lib.g2g_plan_destroy(plan))

    # the scaled form on the same layouts: final = 0.5*final + 2*initial
    scaled = cast = gemr2d = configs = None
    if args.batch and rank == 0 and w.ops is None:
        scaled = run_scaled(lib, w, dI, dF, dts, stream, peak, args.steps // 4 or 1)
        cast = run_cast(lib, dev, stream, peak, args.steps // 4 or 1)
        gemr2d = run_gemr2d(lib, dev, 50)
    if args.batch and rank == 0:
        # the other single-transform configurations, each with its own
        # roofline: block-cyclic double 4096^2 (L2 flushed before every step)
        # and the transposed complex<double> 8192^2
        configs = {}
        for name in ("block_cyclic_f64_4096", "transposed_c128_8192"):
            if name != w.name:
                configs[name] = run_config_leg(lib, name, dev, stream, peak,
                                               max(args.steps, 20),
                                               cpu_reps=args.cpu_reps if ws == 1 else 0)
        # the headline's layouts with op 'T' in float and double (the staged
        # ring of 4- and 8-byte transposed tiles), default tuning, no CPU leg
        for name in ("transposed_random_grid_f32_16384", "transposed_random_grid_f64_16384"):
            if name != w.name:
                configs[name] = run_config_leg(lib, name, dev, stream, peak,
                                               max(args.steps, 20))
        # float 'T' with alpha = 2, beta = 0.5 (the staged ring of scaled
        # transposes: 3x the traffic)
        configs["transposed_random_grid_f32_16384_scaled"] = run_config_leg(
            lib, "transposed_random_grid_f32_16384", dev, stream, peak, max(args.steps, 20),
            ops=[("T", 2.0, 0.5)])

    sharded = None
    if args.batch and rank == 0 and w.ops is None and len(w.inits) == 1:
        sharded = run_sharded_loopback(w, dev, stream, peak, 20)

    batched = serving = None
    if args.batch and rank == 0:
        batched, pool = run_batched(lib, dev, stream, 20, peak,
                                    cpu_reps=args.cpu_reps if ws == 1 else 0)
        if args.serving:
            serving = run_serving(lib, pool, [1000, 5000, 20000], 1.0)
        del pool
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and ws == 1 and args.cpu_reps > 0:
        host_i = [t.cpu().numpy() for t in dev_i]
        host_f = [t.cpu().numpy() for t in dev_f]
        threads = _cpu_threads()
        times, kind, sample = time_cpu_reference(w, args.cpu_reps, threads,
                                                 (host_i, host_f))
        sec = statistics.median(times)
        cpu = {"value": round(w.bytes_moved / sec / 1e9, 4), "unit": UNIT,
               "cores": threads, "kind": kind, "sample": sample}
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_per_step, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": _dtype_name(w),
            "data": "synthetic (seeded random bit patterns, device-resident)",
            "config": _config(w, args), "roofline": roofline, "cpu_baseline": cpu,
            "e2e": e2e, "clocks": clocks, "gpu_launches": args.steps,
            "configs": configs, "sharded_loopback": sharded,
            "batched_stream": batched, "serving": serving,
            "scaled": scaled, "cast": cast, "gemr2d": gemr2d,
            "plan": {"pieces": info.n_pieces, "tiles": info.n_tiles,
                     "create_ms": round(plan_ms, 3), "autotuned": tuned,
                     "default_tuning_kernel_ms": default_ms,
                     "tuning": {k: getattr(info.tuning, k) for k in
                                ("tile_bytes", "tile_dim", "ctas_per_sm", "threads",
                                 "unroll", "stages", "ring", "tile_run", "l2_prefetch",
                                 "tensor_boxes")}},
        }
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _plan_kernel_ms(plan, sp, stream, steps, flush_l2, dev):
    """Mean CUDA-event time of one execution of `plan` (L2 flushed before
    each when the working set fits in it)."""
    import torch
    from grid2grid_gb300 import capi
    lib = capi.load()
    flush = torch.empty(512 * 2**20, dtype=torch.uint8, device=dev) if flush_l2 else None
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    with torch.cuda.stream(stream):
        for _ in range(3):
            capi.check(lib.g2g_plan_execute(plan, sp))
        for a, b in ev:
            if flush is not None:
                flush.zero_()
            a.record(stream)
            capi.check(lib.g2g_plan_execute(plan, sp))
            b.record(stream)
    stream.synchronize()
    return round(statistics.mean(a.elapsed_time(b) for a, b in ev), 5)


def _device_arenas(w, dev, seed):
    import torch
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    di = [torch.randint(0, 256, (L.arena_bytes,), dtype=torch.uint8, device=dev,
                        generator=gen) for L in w.inits]
    df = [torch.randint(0, 256, (L.arena_bytes,), dtype=torch.uint8, device=dev,
                        generator=gen) for L in w.finals]
    return di, df


def _desc_array(layouts, tensors, keep):
    from grid2grid_gb300 import capi
    arr = (capi.LayoutDesc * len(layouts))()
    for k, (L, t) in enumerate(zip(layouts, tensors)):
        d, kk = L.desc(t.data_ptr())
        arr[k] = d
        keep.append(kk)
    return arr


def _time_steps(stream, fn, steps, warmup):
    import torch
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            fn()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
    stream.synchronize()
    return a.elapsed_time(b) / steps


def run_config_leg(lib, name, dev, stream, peak, steps, cpu_reps=0, ops=None):
    """One single-transform configuration, device-resident, plan cached, one
    launch per step timed with CUDA events on the launching stream. Inputs
    smaller than L2 get it flushed before every step, outside the events (a
    512 MiB write, then a 256 MiB read of another buffer). Achieved traffic =
    2 * m * n * sizeof(T) per launch over the mean launch time; `traffic` is
    the DRAM bytes per launch of the committed ncu summary of that kernel."""
    import torch
    from grid2grid_gb300 import capi
    from grid2grid_gb300 import workloads as W
    w = W.BY_NAME[name]()
    if ops is not None:  # the workload's layouts under other ops (alpha, beta)
        w = W.Workload(w.name + "_scaled", w.inits, w.finals, ops, meta=dict(w.meta or {}))
    di, df = _device_arenas(w, dev, 4321)
    keep = []
    n = len(w.inits)
    dI, dF = _desc_array(w.inits, di, keep), _desc_array(w.finals, df, keep)
    dts = (C.c_int * n)(*w.dtypes())
    ops = None if w.ops is None else (capi.Op * n)(*[capi.make_op(*o) for o in w.ops])
    sp = C.c_void_p(stream.cuda_stream)
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create_batch(n, dI, dF, dts, ops, sp, C.byref(plan)))
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    flush = flush_rd = None
    small = w.bytes_moved < 512 * 2**20
    if small:
        flush = torch.empty(512 * 2**20, dtype=torch.uint8, device=dev)
        flush_rd = torch.ones(32 * 2**20, dtype=torch.int64, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    with torch.cuda.stream(stream):
        for _ in range(5):
            capi.check(lib.g2g_plan_execute(plan, sp))
        for k in range(steps):
            if small:
                flush.zero_()
                flush_rd.sum()
            ev[k][0].record(stream)
            capi.check(lib.g2g_plan_execute(plan, sp))
            ev[k][1].record(stream)
    stream.synchronize()
    ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    # plans that qualify also run as 2-D TMA boxes through tensor maps
    # (cp.async.bulk.tensor loads and stores), timed the same way
    boxes = None
    if info.tensor_boxes_ok:
        t = capi.Tuning()
        t.tensor_boxes = 1
        capi.check(lib.g2g_plan_set_tuning(plan, C.byref(t)))
        with torch.cuda.stream(stream):
            for _ in range(5):
                capi.check(lib.g2g_plan_execute(plan, sp))
            for k in range(steps):
                if small:
                    flush.zero_()
                    flush_rd.sum()
                ev[k][0].record(stream)
                capi.check(lib.g2g_plan_execute(plan, sp))
                ev[k][1].record(stream)
        stream.synchronize()
        bms = statistics.mean(a.elapsed_time(b) for a, b in ev)
        bach = info.bytes_min_traffic / (bms * 1e-3) / 1e9
        boxes = {"kernel": "tma_box_kernel (cp.async.bulk.tensor 2-D loads and stores)",
                 "ms_per_step": round(bms, 5),
                 "value": round(w.bytes_moved / (bms * 1e-3) / 1e9, 2), "unit": UNIT,
                 "roofline_frac": round(bach / peak, 4),
                 "traffic": _profile_traffic("tma_box", name)}
    capi.check(lib.g2g_plan_destroy(plan))
    achieved = info.bytes_min_traffic / (ms * 1e-3) / 1e9
    cpu = None
    if cpu_reps > 0:  # the same transform on the host cores, outside the GPU timing
        threads = _cpu_threads()
        times, kind, sample = time_cpu_reference(
            w, cpu_reps, threads, ([t.cpu().numpy() for t in di], [t.cpu().numpy() for t in df]))
        sec = statistics.median(times)
        cpu = {"value": round(w.bytes_moved / sec / 1e9, 4), "unit": UNIT, "cores": threads,
               "kind": kind, "sample": sample}
    del di, df, flush, flush_rd
    torch.cuda.empty_cache()
    return {"workload": w.name, "config": dict(w.meta, ops=w.ops), "ms_per_step": round(ms, 5),
            "cpu_baseline": cpu, "tensor_boxes": boxes,
            "value": round(w.bytes_moved / (ms * 1e-3) / 1e9, 2), "unit": UNIT,
            "steps": steps, "pieces": info.n_pieces, "tiles": info.n_tiles,
            "l2": "flushed before every step (outside the events)" if small
                  else "inputs larger than L2 (no flush)",
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": _profile_traffic("g2g_scatter", w.name),
                         "algorithmic_bytes_per_launch": info.bytes_min_traffic}}


def run_sharded_loopback(w, dev, stream, peak, steps, n_shards=2):
    """The sharded transform's data path on one GPU: the workload's virtual
    ranks split into contiguous halves (two shards), each shard's pack
    (local pieces + send buffer, one launch), the exchange as device-to-device
    copies of the buffer sections (what an all-to-all between two GPUs would
    deliver), each shard's unpack. The link between GPUs is not part of it:
    the time is the HBM work one GPU does for its shard, all shards here."""
    import torch
    from grid2grid_gb300 import exchange as X
    Li, Lf = w.inits[0], w.finals[0]
    P = max(Li.n_ranks, Lf.n_ranks)
    smap = X.contiguous_shards(P, n_shards)
    di, df = _device_arenas(w, dev, 999)
    shards, keep = [], []
    for g in range(n_shards):
        dI, k1 = X.shard_layout(Li, smap, g).desc(di[0].data_ptr())
        dF, k2 = X.shard_layout(Lf, smap, g).desc(df[0].data_ptr())
        keep += [k1, k2]
        shards.append(X.ShardedTransform(dI, dF, Li.dtype, None, smap, g, n_shards, device=dev))

    def exchange():
        for h, dst in enumerate(shards):
            pos = 0
            for g, src in enumerate(shards):
                n = src.send_bytes[h]
                if n:
                    so = sum(src.send_bytes[:h])
                    dst.recv[pos:pos + n].copy_(src.send[so:so + n])
                pos += n
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    t = [0.0, 0.0, 0.0]
    with torch.cuda.stream(stream):
        for k in range(steps + 3):
            ev[0].record(stream)
            for sh in shards:
                sh.pack(stream)
            ev[1].record(stream)
            exchange()
            ev[2].record(stream)
            for sh in shards:
                sh.unpack(stream)
            ev[3].record(stream)
            stream.synchronize()
            if k >= 3:
                for j in range(3):
                    t[j] += ev[j].elapsed_time(ev[j + 1]) / steps
    sent = sum(sum(sh.send_bytes) for sh in shards)
    ms = sum(t)
    for sh in shards:
        sh.close()
    del di, df
    torch.cuda.empty_cache()
    # traffic: every element read and written once (local pieces), or read,
    # packed, copied, unpacked (remote pieces): 2 bytes per byte moved plus
    # 4 per byte sent (pack write + copy read/write + unpack read)
    traffic = 2 * w.bytes_moved + 4 * sent
    return {"workload": w.name, "shards": n_shards, "rank_to_shard": "contiguous halves",
            "bytes_moved": w.bytes_moved, "bytes_exchanged": sent,
            "ms_per_step": round(ms, 4),
            "ms_pack": round(t[0], 4), "ms_exchange_copies": round(t[1], 4),
            "ms_unpack": round(t[2], 4),
            "value": round(w.bytes_moved / (ms * 1e-3) / 1e9, 2), "unit": UNIT,
            "traffic_bytes": traffic,
            "roofline_frac": round(traffic / (ms * 1e-3) / 1e9 / peak, 4),
            "note": "one GPU holds every shard; the inter-GPU link is not measured"}


def run_scaled(lib, w, dI, dF, dts, stream, peak, steps):
    """final = beta*final + alpha*initial with (alpha, beta) = (2, 0.5) on the
    headline layouts (traffic 3x the bytes moved: the destination is read)."""
    from grid2grid_gb300 import capi
    n = len(w.inits)
    ops = (capi.Op * n)(*[capi.make_op("N", 2.0, 0.5) for _ in range(n)])
    sp = C.c_void_p(stream.cuda_stream)
    plan = C.c_void_p()
    capi.check(lib.g2g_plan_create_batch(n, dI, dF, dts, ops, sp, C.byref(plan)))
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    ms = _time_steps(stream, lambda: capi.check(lib.g2g_plan_execute(plan, sp)), steps, 3)
    capi.check(lib.g2g_plan_destroy(plan))
    return {"op": "N, alpha=2, beta=0.5", "ms_per_step": round(ms, 4),
            "value": round(info.bytes_moved / (ms * 1e-3) / 1e9, 2), "unit": UNIT,
            "traffic_bytes": info.bytes_min_traffic,
            "roofline_frac": round(info.bytes_min_traffic / (ms * 1e-3) / 1e9 / peak, 4)}


def run_cast(lib, dev, stream, peak, steps, m=16384):
    """The fused dtype cast on random grid layouts of the headline's kind
    (16 virtual ranks, splits U[1,2048], padded strides): float32 -> float64
    and back. Traffic per element: sizeof(src) + sizeof(dst)."""
    import torch
    from grid2grid_gb300 import capi
    from grid2grid_gb300 import layouts as Ls
    rng = np.random.default_rng(2024)
    L32 = Ls.random_grid_layout(m, m, 16, capi.FLOAT32, rng)
    L64 = Ls.random_grid_layout(m, m, 16, capi.FLOAT64, rng)
    gen = torch.Generator(device=dev)
    gen.manual_seed(99)
    # float32 arena: finite normals; float64 arena: float64 normals
    a32 = torch.randn(L32.arena_bytes // 4, generator=gen, device=dev).view(torch.uint8)
    a64 = torch.randn(L64.arena_bytes // 8, generator=gen, device=dev,
                      dtype=torch.float64).view(torch.uint8)
    keep = []
    d32 = _desc_array([L32], [a32], keep)
    d64 = _desc_array([L64], [a64], keep)
    sp = C.c_void_p(stream.cuda_stream)
    out = {"layouts": "random grids 16384^2, 16 ranks, splits U[1,2048], padded strides"}
    for name, (di, dts, df, dtd) in {"f32_to_f64": (d32, capi.FLOAT32, d64, capi.FLOAT64),
                                     "f64_to_f32": (d64, capi.FLOAT64, d32, capi.FLOAT32)}.items():
        plan = C.c_void_p()
        capi.check(lib.g2g_plan_create_cast(di, dts, df, dtd, None, sp, C.byref(plan)))
        info = capi.PlanInfo()
        capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
        ms_default = _time_steps(stream, lambda: capi.check(lib.g2g_plan_execute(plan, sp)),
                                 steps, 3)
        t = capi.Tuning()  # the plan's knobs picked by the autotuner, as for the main plan
        capi.check(lib.g2g_plan_autotune(plan, sp, 2, C.byref(t)))
        ms = _time_steps(stream, lambda: capi.check(lib.g2g_plan_execute(plan, sp)), steps, 3)
        capi.check(lib.g2g_plan_destroy(plan))
        out[name] = {"ms_per_step": round(ms, 4), "ms_default_tuning": round(ms_default, 4),
                     "value": round(info.bytes_moved / (ms * 1e-3) / 1e9, 2), "unit": UNIT,
                     "traffic_bytes": info.bytes_min_traffic,
                     "roofline_frac": round(info.bytes_min_traffic / (ms * 1e-3) / 1e9 / peak, 4)}
    del a32, a64
    return out


def run_gemr2d(lib, dev, steps, m=4096):
    """The ScaLAPACK-descriptor front end as a caller of p?gemr2d uses it:
    one blocking g2g_gemr2d per step on the block-cyclic double configuration
    (m x m, 32 x 32 blocks -> 128 x 64 blocks on a 2 x 2 grid, lld = local
    rows), per-rank arrays on the device. The call builds both layouts from
    the descriptors, finds the cached plan, launches and synchronises."""
    import torch
    from grid2grid_gb300 import capi

    def desc(mb, nb):
        d = capi.ScalapackDesc()
        d.m, d.n, d.mb, d.nb = m, m, mb, nb
        d.rsrc = d.csrc = 0
        d.nprow, d.npcol, d.row_major = 2, 2, 0
        return d
    loc = m // 2  # local rows and columns of every rank (m a multiple of 256)
    a = [torch.randn(loc * loc, dtype=torch.float64, device=dev) for _ in range(4)]
    b = [torch.zeros(loc * loc, dtype=torch.float64, device=dev) for _ in range(4)]
    pa = (C.c_void_p * 4)(*[t.data_ptr() for t in a])
    pb = (C.c_void_p * 4)(*[t.data_ptr() for t in b])
    lld = (C.c_int32 * 4)(*([loc] * 4))
    da, db = desc(32, 32), desc(128, 64)
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)

    def call():
        capi.check(lib.g2g_gemr2d(m, m, pa, 1, 1, C.byref(da), lld, pb, 1, 1, C.byref(db), lld,
                                  capi.FLOAT64, None, sp))
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        call()
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / steps
    return {"call": "g2g_gemr2d (blocking call latency: descriptors -> cached plan -> launch "
                    "-> synchronise; the 128 MiB working set stays in L2 between calls, so "
                    "this is not an HBM figure -- configs.block_cyclic_f64_4096 is)",
            "config": f"double {m}^2, 32x32 -> 128x64 on 2x2",
            "ms_per_call": round(t * 1e3, 4), "value": round(m * m * 8 / t / 1e9, 2),
            "unit": UNIT, "calls": steps}


def run_cast_only(args):
    import torch
    from grid2grid_gb300 import capi
    lib = capi.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    peak, _ = _peaks()
    print(json.dumps({"cast": run_cast(lib, dev, stream, peak, args.steps)}))
    return 0


def run_batched(lib, dev, stream, steps, peak, cpu_reps=0):
    """uneven_batch_256: 256 redistributions of uneven shapes and dtypes.
    batched = one plan over all pairs (the vector transform), autotuned and
    replayed as a captured CUDA graph: ONE launch per step.
    plain_launches = the same 256 transforms with cached per-transform plans,
    one asynchronous launch each, back to back.
    plain_calls = one blocking g2g_transform call per transform (the
    reference's calling pattern, plans cached).
    multi_plan = the 256 cached plans issued as one launch."""
    from grid2grid_gb300 import capi
    from grid2grid_gb300 import workloads as W
    w = W.uneven_batch(256)
    di, df = _device_arenas(w, dev, 77)
    keep = []
    n = len(w.inits)
    dI, dF = _desc_array(w.inits, di, keep), _desc_array(w.finals, df, keep)
    dts = (C.c_int * n)(*w.dtypes())
    sp = C.c_void_p(stream.cuda_stream)
    plan = C.c_void_p()
    t0 = time.perf_counter()
    capi.check(lib.g2g_plan_create_batch(n, dI, dF, dts, None, sp, C.byref(plan)))
    plan_ms = (time.perf_counter() - t0) * 1e3
    # the batch at the library's default tuning, before autotuning
    ms_bd = _time_steps(stream, lambda: capi.check(lib.g2g_plan_execute(plan, sp)),
                        steps, 3)
    tuned = capi.Tuning()
    capi.check(lib.g2g_plan_autotune(plan, sp, 2, C.byref(tuned)))
    capi.check(lib.g2g_plan_capture_graph(plan, sp))
    info = capi.PlanInfo()
    capi.check(lib.g2g_plan_get_info(plan, C.byref(info)))
    ms_b = _time_steps(stream, lambda: capi.check(lib.g2g_plan_execute(plan, sp)),
                       steps, 3)
    plans = (C.c_void_p * n)()
    t0 = time.perf_counter()
    for k in range(n):
        p = C.c_void_p()
        capi.check(lib.g2g_plan_create(C.byref(dI[k]), C.byref(dF[k]), dts[k], None, sp,
                                       C.byref(p)))
        plans[k] = p.value
    plans_ms = (time.perf_counter() - t0) * 1e3

    def plain():
        for k in range(n):
            capi.check(lib.g2g_plan_execute(plans[k], sp))
    ms_p = _time_steps(stream, plain, max(2, steps // 4), 1)
    ms_m = _time_steps(stream, lambda: capi.check(lib.g2g_plans_execute(n, plans, sp)),
                       steps, 2)
    # the same tuning policy on both sides: every per-transform plan under the
    # knobs the autotuner picked for the batch
    for k in range(n):
        capi.check(lib.g2g_plan_set_tuning(plans[k], C.byref(tuned)))
    ms_pt = _time_steps(stream, plain, max(2, steps // 4), 1)

    # the reference's calling pattern: one blocking transform call per pair
    # (one-shot API; its plans are cached after the first pass)
    def calls():
        for k in range(n):
            capi.check(lib.g2g_transform(C.byref(dI[k]), C.byref(dF[k]), dts[k], None, sp))
    calls()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        calls()
    ms_c = (time.perf_counter() - t0) * 1e3 / reps
    capi.check(lib.g2g_plan_cache_clear())
    for k in range(n):
        capi.check(lib.g2g_plan_destroy(plans[k]))
    capi.check(lib.g2g_plan_destroy(plan))
    b = w.bytes_moved
    # the same 256 transforms on the host cores (one pass after a warm-up)
    cpu = None
    if cpu_reps > 0:
        threads = _cpu_threads()
        times, kind, sample = time_cpu_reference(
            w, 1, threads, ([t.cpu().numpy() for t in di], [t.cpu().numpy() for t in df]))
        cpu = {"value": round(b / statistics.median(times) / 1e9, 4), "unit": UNIT,
               "cores": threads, "kind": kind, "sample": sample}
    return {
        "workload": w.name, "bytes_per_step": b, "pieces": info.n_pieces,
        "tiles": info.n_tiles,
        "batched": {"value": round(b / (ms_b * 1e-3) / 1e9, 2), "unit": UNIT,
                    "ms_per_step": round(ms_b, 4), "launches_per_step": 1,
                    "roofline_frac": round(info.bytes_min_traffic / (ms_b * 1e-3) / 1e9 / peak, 4),
                    "plan_ms": round(plan_ms, 1),
                    "tuning": {k: getattr(tuned, k) for k in
                               ("tile_bytes", "tile_dim", "ctas_per_sm", "threads", "unroll",
                                "stages", "ring", "tile_run", "l2_prefetch")},
                    "graph": True},
        "batched_default_tuning": {"value": round(b / (ms_bd * 1e-3) / 1e9, 2), "unit": UNIT,
                                   "ms_per_step": round(ms_bd, 4), "launches_per_step": 1,
                                   "graph": False},
        "plain_launches": {"value": round(b / (ms_p * 1e-3) / 1e9, 2), "unit": UNIT,
                           "ms_per_step": round(ms_p, 4), "launches_per_step": n,
                           "plan_ms_total": round(plans_ms, 1),
                           "tuning": "each plan's default"},
        "plain_launches_batch_tuning": {"value": round(b / (ms_pt * 1e-3) / 1e9, 2),
                                        "unit": UNIT, "ms_per_step": round(ms_pt, 4),
                                        "launches_per_step": n,
                                        "tuning": "the batch's autotuned knobs"},
        "multi_plan_launch": {"value": round(b / (ms_m * 1e-3) / 1e9, 2), "unit": UNIT,
                              "ms_per_step": round(ms_m, 4), "launches_per_step": 1},
        "plain_calls": {"value": round(b / (ms_c * 1e-3) / 1e9, 2), "unit": UNIT,
                        "ms_per_step": round(ms_c, 4), "launches_per_step": n,
                        "path": "256 blocking g2g_transform calls (plans cached)"},
        "speedup_batched_vs_plain_launches": round(ms_p / ms_b, 3),
        "bound": _batch_bound(w, ms_b, ms_p, peak),
        "speedup_same_tuning": {"default": round(ms_p / ms_bd, 3),
                                "autotuned": round(ms_pt / ms_b, 3)},
        "speedup_batched_vs_plain_calls": round(ms_c / ms_b, 3),
        "cpu_baseline": cpu,
    }, (w, di, df, dI, dF, dts, keep)


def _batch_bound(w, ms_b, ms_p, peak):
    """What the layout mix allows: the sector-level DRAM traffic floor of the
    batch (every column's 32-byte sectors once, plus the fills of partial
    destination sectors next to padding) at the measured copy peak, and the
    speed-up over the plain launches that a batch at that floor would reach."""
    from grid2grid_gb300 import workloads as W
    t = W.sector_traffic(w)
    floor_ms = t["total"] / (peak * 1e9) * 1e3
    return {"sector_traffic_bytes": t["total"], "algorithmic_bytes": t["algorithmic"],
            "traffic_ratio": round(t["total"] / t["algorithmic"], 4),
            "ms_at_copy_peak": round(floor_ms, 4),
            "max_speedup_vs_plain_launches": round(ms_p / floor_ms, 3),
            "copy_peak_fraction_for_3x": round(t["total"] / (ms_p / 3 * 1e-3) / 1e9 / peak, 4),
            "batched_frac_of_floor": round(floor_ms / ms_b, 4)}


def run_serving(lib, pool, rates, duration_s, seed=5):
    """Open-loop Poisson arrivals of requests drawn from the uneven batch
    pool (plans cached), through the continuous-batching server and through
    plain per-request launches (max_batch_requests = 1, one launch in
    flight). Latency = completion - arrival."""
    from grid2grid_gb300 import capi
    w, di, df, dI, dF, dts, keep = pool
    n = len(w.inits)
    rng = np.random.default_rng(seed)
    servers = {}
    for mode, cfg in (("continuous", dict(max_batch_requests=256, max_launches_in_flight=3)),
                      ("plain", dict(max_batch_requests=1, max_launches_in_flight=1))):
        c = capi.ServerConfig()
        c.hbm_budget_bytes = 120 * 10**9
        for k, v in cfg.items():
            setattr(c, k, v)
        srv = C.c_void_p()
        capi.check(lib.g2g_server_create(C.byref(c), C.byref(srv)))
        servers[mode] = srv
    out = {"budget_bytes": 120 * 10**9, "duration_s": duration_s, "rates": {}}
    try:
        for mode, srv in servers.items():
            # warm the plan caches (a burst of every pair), then the launch
            # path at a low rate (0.2 s at the first rate), both discarded
            idx = (C.c_int32 * n)(*range(n))
            arr = (C.c_double * n)(*([0.0] * n))
            times = (capi.RequestTimes * n)()
            capi.check(lib.g2g_server_replay(srv, n, dI, dF, dts, None, n, idx, arr, times))
            Nw = max(1, int(rates[0] * 0.2))
            warr = np.cumsum(rng.exponential(1.0 / rates[0], size=Nw)).astype(np.float64)
            wpick = rng.integers(0, n, size=Nw).astype(np.int32)
            wtimes = (capi.RequestTimes * Nw)()
            capi.check(lib.g2g_server_replay(srv, n, dI, dF, dts, None, Nw,
                                             wpick.ctypes.data_as(C.POINTER(C.c_int32)),
                                             warr.ctypes.data_as(C.POINTER(C.c_double)),
                                             wtimes))
        for rate in rates:
            N = int(rate * duration_s)
            arrivals = np.cumsum(rng.exponential(1.0 / rate, size=N))
            pick = rng.integers(0, n, size=N).astype(np.int32)
            res = {}
            for mode, srv in servers.items():
                idx = pick.ctypes.data_as(C.POINTER(C.c_int32))
                arr = arrivals.astype(np.float64)
                times = (capi.RequestTimes * N)()
                capi.check(lib.g2g_server_replay(srv, n, dI, dF, dts, None, N, idx,
                                                 arr.ctypes.data_as(C.POINTER(C.c_double)),
                                                 times))
                t = np.ctypeslib.as_array(times)
                lat = (t["complete_ns"] - t["submit_ns"]) / 1e3
                span = (t["complete_ns"].max() - t["submit_ns"].min()) / 1e9
                res[mode] = {"p50_us": round(float(np.percentile(lat, 50)), 1),
                             "p99_us": round(float(np.percentile(lat, 99)), 1),
                             "mean_us": round(float(lat.mean()), 1),
                             "GBps": round(float(t["bytes"].sum()) / span / 1e9, 2),
                             "mean_batch": round(float(t["batch_size"].mean()), 2),
                             "requests": N}
            out["rates"][str(rate)] = res
    finally:
        for srv in servers.values():
            capi.check(lib.g2g_server_destroy(srv))
    return out


def run_e2e(lib, w, dev_i, dev_f, steps, stream, ws):
    """Host-buffer transforms, every step's copies inside the timing.

    sequential: per step, H2D of the initial layout's arena from pinned
      memory, one-shot g2g_transform_batch (blocking; plan cached after the
      first call), D2H of the final layout's arena.
    pipelined (the reported value): the same per-step work on two streams
      with two arena sets, so step k+1's H2D overlaps step k's D2H on the
      host link; each step runs g2g_plan_execute of its set's plan. Five
      trials of `steps` steps; the median trial is reported (the host link
      is shared with other work on the node, and single trials have run
      twice as long as their neighbours).
    The device copy of the final arena mirrors the host one (same padding
    bytes), so copying it back leaves the host padding unchanged."""
    import torch
    from grid2grid_gb300 import capi
    n = len(w.inits)
    dts = (C.c_int * n)(*w.dtypes())
    ops = None
    if w.ops is not None:
        ops = (capi.Op * n)(*[capi.make_op(*o) for o in w.ops])
    keep = []
    sets = []
    for k in range(2):
        di = dev_i if k == 0 else [torch.empty_like(t) for t in dev_i]
        df = dev_f if k == 0 else [t.clone() for t in dev_f]
        hi = [t.cpu().pin_memory() for t in dev_i]
        hf = [t.cpu().pin_memory() for t in dev_f]
        dI, dF = _desc_array(w.inits, di, keep), _desc_array(w.finals, df, keep)
        st = torch.cuda.Stream(device=dev_i[0].device)
        sets.append(dict(di=di, df=df, hi=hi, hf=hf, dI=dI, dF=dF, stream=st))
    h2d = sum(t.numel() for t in sets[0]["hi"])
    d2h = sum(t.numel() for t in sets[0]["hf"])

    # sequential, through the one-shot call
    s0 = sets[0]
    sp0 = C.c_void_p(s0["stream"].cuda_stream)

    def seq_step():
        with torch.cuda.stream(s0["stream"]):
            for d, h in zip(s0["di"], s0["hi"]):
                d.copy_(h, non_blocking=True)
        capi.check(lib.g2g_transform_batch(n, s0["dI"], s0["dF"], dts, ops, sp0))
        with torch.cuda.stream(s0["stream"]):
            for d, h in zip(s0["df"], s0["hf"]):
                h.copy_(d, non_blocking=True)
        s0["stream"].synchronize()
    seq_step()  # warm-up (plans the transform once)
    _barrier(ws)
    t0 = time.perf_counter()
    for _ in range(steps):
        seq_step()
    t_seq = _allreduce_max((time.perf_counter() - t0) / steps, ws)

    # pipelined, two steps in flight
    plans = []
    for sset in sets:
        p = C.c_void_p()
        capi.check(lib.g2g_plan_create_batch(n, sset["dI"], sset["dF"], dts, ops,
                                             C.c_void_p(sset["stream"].cuda_stream),
                                             C.byref(p)))
        plans.append(p)

    def pipe_step(k):
        sset = sets[k % 2]
        st = sset["stream"]
        with torch.cuda.stream(st):
            for d, h in zip(sset["di"], sset["hi"]):
                d.copy_(h, non_blocking=True)
            capi.check(lib.g2g_plan_execute(plans[k % 2], C.c_void_p(st.cuda_stream)))
            for d, h in zip(sset["df"], sset["hf"]):
                h.copy_(d, non_blocking=True)
    # warm-up: a full trial's worth of steps (the first passes over the pinned
    # arenas run measurably slower on the host link)
    for k in range(max(2, steps)):
        pipe_step(k)
    torch.cuda.synchronize()
    trials = []
    for _ in range(5):  # the host link varies between runs: median of 5 trials
        _barrier(ws)
        t0 = time.perf_counter()
        for k in range(steps):
            pipe_step(k)
        torch.cuda.synchronize()
        trials.append(_allreduce_max((time.perf_counter() - t0) / steps, ws))
    t_pipe = sorted(trials)[2]
    for p in plans:
        capi.check(lib.g2g_plan_destroy(p))

    # the host-link bound of the same step: its copies alone, same streams
    def copy_step(k):
        sset = sets[k % 2]
        with torch.cuda.stream(sset["stream"]):
            for d, h in zip(sset["di"], sset["hi"]):
                d.copy_(h, non_blocking=True)
            for d, h in zip(sset["df"], sset["hf"]):
                h.copy_(d, non_blocking=True)
    ctrials = []
    for _ in range(3):
        _barrier(ws)
        t0 = time.perf_counter()
        for k in range(steps):
            copy_step(k)
        torch.cuda.synchronize()
        ctrials.append(_allreduce_max((time.perf_counter() - t0) / steps, ws))
    t_copies = min(ctrials) # the bound: the fastest the link carried the step's copies

    # zero copy: the layouts point at the pinned host arenas themselves; the
    # kernel reads and writes them over the host link, no staging copies
    s0 = sets[0]
    zI, zF = _desc_array(w.inits, s0["hi"], keep), _desc_array(w.finals, s0["hf"], keep)
    zp = C.c_void_p()
    capi.check(lib.g2g_plan_create_batch(n, zI, zF, dts, ops, sp0, C.byref(zp)))
    for _k in range(max(1, steps)):
        capi.check(lib.g2g_plan_execute(zp, sp0))
    s0["stream"].synchronize()
    ztrials = []
    for _ in range(3):
        _barrier(ws)
        t0 = time.perf_counter()
        for _k in range(steps):
            capi.check(lib.g2g_plan_execute(zp, sp0))
        s0["stream"].synchronize()
        ztrials.append(_allreduce_max((time.perf_counter() - t0) / steps, ws))
    capi.check(lib.g2g_plan_destroy(zp))
    t_zero = sorted(ztrials)[1]
    zero = {"value": round(w.bytes_moved * ws / t_zero / 1e9, 3), "unit": UNIT,
            "ms_per_step": round(t_zero * 1e3, 3),
            "trials_ms_per_step": [round(t * 1e3, 3) for t in ztrials],
            "h2d_bytes_per_step": int(w.bytes_moved), "d2h_bytes_per_step": int(w.bytes_moved),
            "path": "g2g_plan_execute on layouts in pinned host memory (the kernel reads and "
                    "writes the host arenas over the host link)"}
    return {"value": round(w.bytes_moved * ws / t_pipe / 1e9, 3), "unit": UNIT,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": round(t_pipe * 1e3, 3), "steps": steps,
            "trials_ms_per_step": [round(t * 1e3, 3) for t in trials],
            "path": "pinned host arenas -> H2D -> g2g_plan_execute -> D2H, two steps in "
                    "flight on two streams",
            "copies_only": {"ms_per_step": round(t_copies * 1e3, 3),
                            "trials_ms_per_step": [round(t * 1e3, 3) for t in ctrials],
                            "link_gbs": round((h2d + d2h) / t_copies / 1e9, 1),
                            "frac": round(t_copies / t_pipe, 4),
                            "path": "the same H2D and D2H copies without the transform "
                                    "(the host-link bound of a step)"},
            "sequential": {"value": round(w.bytes_moved * ws / t_seq / 1e9, 3),
                           "ms_per_step": round(t_seq * 1e3, 3),
                           "path": "pinned host arenas -> H2D -> g2g_transform_batch "
                                   "(blocking, plan cached) -> D2H"},
            "zero_copy": zero}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="random_grid_f32_16384")
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--cpu-reps", type=int, default=2)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="time the main plan at the library's default tuning instead of "
                         "the knobs its autotuner picks")
    ap.add_argument("--tuning", default="", metavar="K=V,...",
                    help="g2g_tuning fields for the main plan (e.g. stages=3 for the "
                         "TMA-staged kernel)")
    ap.add_argument("--alpha-beta", type=lambda v: tuple(float(x) for x in v.split(",")),
                    default=None, metavar="A,B",
                    help="time final = B*final + A*op(initial) on the workload instead "
                         "of its plain transform (the scaled kernel instances)")
    ap.add_argument("--cast-only", action="store_true",
                    help="time only the fused dtype casts (float32 <-> float64 on random "
                         "grids) and print their figures (the cast kernel instances)")
    ap.add_argument("--no-batch", dest="batch", action="store_false",
                    help="skip the 256-transform batched stream")
    ap.add_argument("--no-serving", dest="serving", action="store_false",
                    help="skip the Poisson serving measurement")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.cast_only:
        return run_cast_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
