"""Benchmark of the sync-free triangular solve on GB300.

Workload ("step"): the plain FP64 sync-free solves of the deep-vs-wide pair,
rhs = 1, forward and backward (upper = L^T):
  (a) lower triangle of the 5-point Laplacian on a 1414 x 1414 mesh
      (n = 1,999,396, 5,995,360 stored entries, 2,827 level sets);
  (b) random lower triangle, n = 4,194,304, power-law column counts
      (alpha 2.1, cap 1000) scaled to ~38M stored entries, rows within
      j+1..j+50,000.
One step = 4 solves ((a) fwd, (a) bwd, (b) fwd, (b) bwd) on synthetic seeded
inputs. The metric is effective GB/s: algorithmic bytes of each solve,
B = 4(n+1) + nnz(4+8) + 2*8n (column pointers, row indices, values, read b,
write x), summed over the step and divided by the step's device time. L2 is
flushed (256 MiB write) before every solve, outside the timed events.

Arms:
  default          the library (libsptrsv_gb300.so) on cuda:LOCAL_RANK.
  --impl reference the reference's serial CPU executor for this path (the
                   oracle: a C restatement of SpTRSV_cuda/sptrsv_syncfree_serialref.h,
                   or the reference build where it exists), the four solves of a
                   step run concurrently on four host threads.
Multi-GPU: every rank solves the same workload independently (replicas);
the batch workload instead shards its systems over the ranks (nnz-balanced)
and the multi_rhs workload its right-hand-side columns (contiguous slices).
Profiling runs: --scale shrinks the systems, --cases picks a subset, and
--opt KEY=VALUE fixes a solver option (the autotuner is then skipped).

Other workloads (--workload; each prints one JSON line of its own metric):
  multi_rhs  n = 1,000,000, Poisson(9) off-diagonals in a band of 20,000,
             rhs in {1, 16, 64}, B ~ N(0,1) column-major: plain FP64 solve vs
             FP32 storage/solve + FP64-residual refinement; forward error vs
             the FP64 oracle.
  batch      512 independent systems (even lower, odd upper), n log-uniform on
             [1e3, 2e5], stored entries per column U{3..20}, band U[100, 1e4],
             rhs = 4: one batched FP32+refinement launch sequence vs 512
             per-system plain FP64 launches; systems solved per second.
  adjoint    the multi_rhs matrix, rhs = 8, FP64, loss = sum(w * x):
             forward + adjoint (fused value gradient) time over forward time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "benchmark-sptrsv_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "SpTRSV effective GB/s (FP64 sync-free solve, rhs=1, Laplacian-2M + power-law-4M, fwd+bwd)"
WORKLOAD = "laplace1414_2M + powerlaw_4M, FP64, rhs=1, forward+backward (4 solves per step)"


def bytes_pass(n: int, nnz: int, rhs: int = 1, sv: int = 8, sx: int = 8) -> int:
    return 4 * (n + 1) + nnz * (4 + sv) + n * rhs * 2 * sx


CASE_NAMES = ("laplace_fwd", "laplace_bwd", "powerlaw_fwd", "powerlaw_bwd")


def make_cases(scale: float = 1.0, only=None):
    from sptrsv_gb300 import matgen
    if scale == 1.0:
        lap = matgen.system_laplace_2m(lower=True)
        pl = matgen.system_powerlaw_4m(seed=1, lower=True)
    else:   # reduced copies of the same systems (profiling runs)
        lap = matgen.laplace2d_lower(max(8, int(round(1414 * scale ** 0.5))))
        pl = matgen.system_powerlaw_4m(seed=1, lower=True, n=max(1024, int(matgen.POWER_LAW_N * scale)),
                                       target_nnz=max(4096, int(40_000_000 * scale)))
    cases = []
    for name, m in (("laplace_fwd", lap), ("laplace_bwd", lap.transpose()),
                    ("powerlaw_fwd", pl), ("powerlaw_bwd", pl.transpose())):
        if only and name not in only:
            continue
        x_true = np.ones(m.n)
        b = m.matvec(x_true)
        cases.append(dict(name=name, m=m, b=b))
    return cases


def workload_config(args, world: int) -> dict:
    """The `config` of both arms' JSON lines (identical, so the lines compare)."""
    return {"workload": WORKLOAD if args.scale == 1.0 else f"{WORKLOAD}, sizes x{args.scale}", "rhs": 1,
            "dtype": "f64", "parallelism": f"replicas x{world}" if world > 1 else "one device",
            "mode": "replicas" if world > 1 else "single",
            "l2": "GPU arm: flushed (256 MiB write) before every solve and before every end-to-end step, "
                  "outside the timed events; CPU arm: inputs larger than the host caches for the power-law system"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ reference (CPU) arm
def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle
    imp = oracle.ref() or oracle.port()
    kind = "reference" if imp.kind == "ref" else "port"
    cases = make_cases(args.scale)
    degs = [imp.analyser(c["m"].row_idx, c["m"].n) for c in cases]
    total_bytes = sum(bytes_pass(c["m"].n, c["m"].nnz) for c in cases)

    def one(i):
        c = cases[i]
        m = c["m"]
        return imp.executor(m.col_ptr, m.row_idx, m.val, degs[i], m.n, m.substitution, 1, c["b"])

    threads = len(cases)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for _ in range(args.warmup):
            list(ex.map(one, range(len(cases))))
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            xs = list(ex.map(one, range(len(cases))))
            times.append(time.perf_counter() - t0)
    err = max(float(np.max(np.abs(x - 1.0))) for x in xs)
    ms = 1e3 * sum(times) / len(times)
    value = total_bytes / (ms * 1e-3) / 1e9
    sample = f"{args.steps} steps of the full workload (4 serial solves per step, one per thread)"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(args, world),
        "cpu_baseline": {"value": round(value, 4), "unit": "GB/s", "cores": threads, "kind": kind,
                         "sample": sample, "host": host_info()},
        "e2e": {"value": round(value, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "max_abs_err_vs_ones": err,
    }
    print(json.dumps(line), flush=True)
    return 0


def host_info() -> dict:
    """The host the CPU arms ran on: architecture, logical cores, CPU model
    (/proc/cpuinfo 'model name', or the Arm implementer/part codes)."""
    import platform
    model = ""
    try:
        fields = {}
        for ln in open("/proc/cpuinfo"):
            if ":" in ln:
                k, v = ln.split(":", 1)
                fields.setdefault(k.strip(), v.strip())
        model = fields.get("model name") or (
            f"implementer {fields.get('CPU implementer', '?')} part {fields.get('CPU part', '?')}"
            if "CPU part" in fields else "")
    except OSError:
        pass
    return {"machine": platform.machine(), "nproc": os.cpu_count(), "cpu_model": model or platform.processor()}


def cpu_baseline_sample(cases):
    """Serial oracle on the host (1 core), bounded sample: each case solved until ~4 s each."""
    from oracle import oracle
    imp = oracle.ref() or oracle.port()
    kind = "reference" if imp.kind == "ref" else "port"
    tot_bytes, tot_s, solves = 0, 0.0, 0
    for c in cases:
        m = c["m"]
        deg = imp.analyser(m.row_idx, m.n)
        t_case = 0.0
        while t_case < 4.0:
            t0 = time.perf_counter()
            imp.executor(m.col_ptr, m.row_idx, m.val, deg, m.n, m.substitution, 1, c["b"])
            dt = time.perf_counter() - t0
            t_case += dt
            tot_s += dt
            tot_bytes += bytes_pass(m.n, m.nnz)
            solves += 1
    return {"value": round(tot_bytes / tot_s / 1e9, 4), "unit": "GB/s", "cores": 1, "kind": kind,
            "sample": f"{solves} serial FP64 solves over the 4 workload systems (~4 s each), 1 thread",
            "host": host_info()}


# ------------------------------------------------------------------ GPU arm
# DRAM bytes per stored entry of the split-list executor on the power-law
# backward system: ncu capture of the 1/4-size case (156.0 MB for 9,474,199
# stored entries; traffic grows with the stored entries), scaled to a launch.
TRAFFIC_PER_ENTRY = {"powerlaw_bwd": (145.447680e6 + 10.590208e6) / 9474199}
TRAFFIC_SOURCE = ("ncu --set full capture of k_pull_wsync_split on powerlaw_bwd at 1/4 size, scaled by stored "
                  "entries (profiles/k_pull_wsync_split_powerlaw_bwd.md)")


def traffic_bytes(case):
    per = TRAFFIC_PER_ENTRY.get(case["name"])
    return int(round(per * case["m"].nnz)) if per else None


def reference_scheme_ms(cases, dev, reps: int = 3) -> dict:
    """Median device time of the reference's executor scheme (kernel-level surface) per case."""
    import torch

    from sptrsv_gb300 import OPT_WARP_AUTO, analyser, executor
    out = {}
    for c in cases:
        m = c["m"]
        cp = torch.from_numpy(m.col_ptr).to(dev)
        ri = torch.from_numpy(m.row_idx).to(dev)
        va = torch.from_numpy(m.val).to(dev)
        deg0 = torch.zeros(m.n, dtype=torch.int32, device=dev)
        analyser(ri, m.n, m.nnz, deg0)
        deg = torch.empty_like(deg0)
        left = torch.zeros(m.n, dtype=torch.float64, device=dev)
        b = c["b_dev"]
        x = torch.empty_like(b)
        ts = []
        for _ in range(reps + 1):
            deg.copy_(deg0)
            left.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            executor(cp, ri, va, deg, left, m.n, m.substitution, 1, OPT_WARP_AUTO, b, x)
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        if float((x - 1.0).abs().max()) > 1e-9:
            raise RuntimeError(f"reference scheme gave a wrong solution on {c['name']}")
        out[c["name"]] = statistics.median(ts[1:])
    return out


# Hardware hop latencies measured on GB300 by a stand-alone probe (figures in
# profiles/machine_probe_gb300.md): one-way flag hop SM -> SM with a relaxed
# store and a relaxed poll, 303 ns (627 cycles; 464 ns on another box), and a
# warp -> warp hop through shared memory inside one CTA, 196 cycles.
HW_HOP_GLOBAL_NS = (303.0, 464.0)
HW_HOP_SMEM_CYCLES = 196.0


def hop_latency(dev, n: int = 8192, reps: int = 9) -> dict:
    """Per-hop latency of this library's executor, measured on a chain (unknown j
    feeds j+1 only, n levels): one unknown per chunk puts every hop through global
    memory (publish, L2, poll by another CTA); one chunk for the whole chain puts
    every hop through the CTA's shared memory. nlevels x t_hop is the floor of a
    solve whose hops all take that path."""
    import torch

    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.chain(n)
    b = torch.from_numpy(m.matvec(np.ones(n))).to(dev)
    out = {}
    for name, chunk in (("global", 1), ("smem", n)):
        s = SyncFreeSolver(m.col_ptr, m.row_idx, n, 0, values=m.val, schedule=2, staged=False, warp_sync=True,
                           order_block=2**31 - 1, chunk=chunk, sync_check=False)
        x = s.solve(b)
        ms = _timed(lambda: s.solve(b, out=x), reps)
        s.check()
        out[name] = 1e3 * ms / n
        s.close()
    return out


def run_gpu(args, world, rank, local):
    import torch

    from sptrsv_gb300 import SyncFreeSolver

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    cases = make_cases(args.scale, args.cases)
    solvers = []
    tuned = {}
    for c in cases:
        m = c["m"]
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, sync_check=True,
                           profile=True, **args.solver_kw)
        c["solver"] = s
        c["b_dev"] = torch.from_numpy(c["b"]).to(dev)
        c["x_dev"] = torch.empty_like(c["b_dev"])
        c["bytes"] = bytes_pass(m.n, m.nnz)
        if not args.no_tune and not args.solver_kw:
            # the library's autotuner picks the executor configuration for this system (setup, untimed)
            tuned[c["name"]] = s.tune(c["b_dev"], values=torch.from_numpy(m.val).to(dev), reps=3)
        s.set_option(7, 0)   # asynchronous solves inside the timed region
        solvers.append(s)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def step(record):
        for c in cases:
            flush.fill_(c["bytes"] & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            c["solver"].solve(c["b_dev"], out=c["x_dev"])
            e1.record(stream)
            if record is not None:
                record.append((c["name"], e0, e1, c))

    for _ in range(args.warmup):
        step(None)
    for s in solvers:
        s.check()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.2)
    rec = []
    exec_ms = {c["name"]: [] for c in cases}
    t_wall0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")   # profilers select the timed launches by this range
    for _ in range(args.steps):
        step(rec)
        for c in cases:   # executor-kernel events of this step (waits for the kernel)
            exec_ms[c["name"]].append(c["solver"].exec_ms())
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    t_wall = time.perf_counter() - t_wall0
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    for s in solvers:
        s.check()
    per_case = {c["name"]: [] for c in cases}
    for name, e0, e1, c in rec:
        per_case[name].append(e0.elapsed_time(e1))
    step_ms = sum(statistics.mean(v) for v in per_case.values())
    if pg:
        t = torch.tensor([step_ms], dtype=torch.float64, device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        step_ms = float(t.item())
    total_bytes = sum(c["bytes"] for c in cases)
    value = world * total_bytes / (step_ms * 1e-3) / 1e9

    # correctness of the timed outputs (x_true = 1)
    errs = {c["name"]: float((c["x_dev"] - 1.0).abs().max()) for c in cases}

    # end to end through the public API: pinned host b -> device, solve, device -> host x.
    # Copies run on a second stream so that they overlap the other systems' solves
    # (each solve waits for its own b; each x read-back waits for its own solve).
    h2d = d2h = 0
    for c in cases:
        c["b_host"] = torch.from_numpy(c["b"]).pin_memory()
        c["x_host"] = torch.empty_like(c["b_host"]).pin_memory()
    copy_stream = torch.cuda.Stream(device=dev)
    # the first b copy and the last x read-back cannot overlap a solve: put the
    # systems with the smallest vectors at the two ends
    by_size = sorted(cases, key=lambda c: c["b"].size)
    e2e_order = by_size[0::2] + by_size[1::2][::-1]
    e2e_ms = []
    for it in range(args.warmup + args.steps):
        flush.fill_(it & 0xFF)   # cold L2, as in the device-timed loop (outside the timed region)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        arrived = []
        with torch.cuda.stream(copy_stream):
            for c in e2e_order:
                c["b_dev"].copy_(c["b_host"], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy_stream)
                arrived.append(ev)
        for c, ev in zip(e2e_order, arrived):
            stream.wait_event(ev)
            c["solver"].solve(c["b_dev"], out=c["x_dev"])
            solved = torch.cuda.Event()
            solved.record(stream)
            copy_stream.wait_event(solved)
            with torch.cuda.stream(copy_stream):
                c["x_host"].copy_(c["x_dev"], non_blocking=True)
        torch.cuda.synchronize()
        if it >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    for c in cases:
        h2d += c["b_host"].numel() * 8
        d2h += c["x_host"].numel() * 8
    e2e_step = statistics.mean(e2e_ms)
    if pg:
        t = torch.tensor([e2e_step], dtype=torch.float64, device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_step = float(t.item())
    e2e_val = world * total_bytes / (e2e_step * 1e-3) / 1e9

    # the reference's own GPU scheme on the same systems (outside the timed region):
    # warp per column, in-degree countdown counters and atomic partial sums
    # (SpTRSV_cuda/sptrsv_syncfree_cuda.h:8-107), restated with ticket order and
    # bounded waits, through the kernel-level C-ABI surface
    ref_scheme = reference_scheme_ms(cases, dev) if not args.no_ref_scheme else {}

    # latency floor: nlevels x the per-hop latency of the path the schedule's hops take
    # (global memory in level order, shared memory inside the blocks of a blocked order)
    hop = hop_latency(dev)
    # roofline of the dominant kernel (the executor on the case with the largest share)
    peak, peak_kind = read_peaks()
    dom = max(cases, key=lambda c: statistics.mean(exec_ms[c["name"]]))
    dom_ms = statistics.mean(exec_ms[dom["name"]])
    achieved = dom["bytes"] / (dom_ms * 1e-3) / 1e9
    info = {c["name"]: c["solver"].info() for c in cases}
    details = {}
    for c in cases:
        ms = statistics.mean(per_case[c["name"]])
        ems = statistics.mean(exec_ms[c["name"]])
        details[c["name"]] = {
            "n": c["m"].n, "nnz": c["m"].nnz, "nlevels": info[c["name"]]["nlevels"],
            "solve_ms": round(ms, 4), "exec_kernel_ms": round(ems, 4),
            "gbs": round(c["bytes"] / (ms * 1e-3) / 1e9, 2),
            "roofline_frac": round(c["bytes"] / (ems * 1e-3) / 1e9 / peak, 5),
            "us_per_level": round(1e3 * ems / max(info[c["name"]]["nlevels"], 1), 3),
            "max_abs_err": errs[c["name"]], "analysis_ms": round(info[c["name"]]["analysis_ms"], 2),
        }
        blocked = info[c["name"]]["order_block"] < c["m"].n
        floor_ms = info[c["name"]]["nlevels"] * hop["smem" if blocked else "global"] * 1e-3
        details[c["name"]]["latency_floor_ms"] = round(floor_ms, 4)
        details[c["name"]]["floor_path"] = "shared memory (blocked order)" if blocked else "global memory (level order)"
        details[c["name"]]["exec_over_floor"] = round(ems / floor_ms, 2) if floor_ms > 0 else None
        # the same floor from the hardware hop alone (no executor loop around it)
        sm_mhz = clock_info.get("sm_mhz") or 2070.0
        hw_ns = ((HW_HOP_SMEM_CYCLES / sm_mhz * 1e3,) * 2) if blocked else HW_HOP_GLOBAL_NS
        hw_ms = [info[c["name"]]["nlevels"] * h * 1e-6 for h in hw_ns]
        details[c["name"]]["hw_hop_floor_ms"] = [round(v, 4) for v in hw_ms]
        details[c["name"]]["exec_over_hw_hop_floor"] = [round(ems / v, 2) for v in hw_ms[::-1]]
        if c["name"] in ref_scheme:
            details[c["name"]]["reference_scheme_ms"] = round(ref_scheme[c["name"]], 4)
            details[c["name"]]["speedup_vs_reference_scheme"] = round(ref_scheme[c["name"]] / ms, 2)
    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return 0
    cpu = cpu_baseline_sample(cases) if (world == 1 and not args.no_cpu_baseline) else None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators, x_true = 1)",
        "config": workload_config(args, world),
        "solver": {"settings": args.solver_kw or ("defaults" if args.no_tune else "autotuned per system"),
                   "tuned": tuned},
        "per_rank_value": round(total_bytes / (step_ms * 1e-3) / 1e9, 3),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 3), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": traffic_bytes(dom),
                     "traffic_unit": "bytes per launch (DRAM read + write)",
                     "traffic_source": TRAFFIC_SOURCE if traffic_bytes(dom) else None,
                     "kernel": f"executor on {dom['name']}", "peak_source": peak_kind},
        "latency_floor": {"t_hop_global_us": round(hop["global"], 4), "t_hop_smem_us": round(hop["smem"], 4),
                          "floor_ms_per_step": round(sum(d["latency_floor_ms"] for d in details.values()), 4),
                          "how": "chain of 8,192 unknowns: one unknown per chunk (every hop through global "
                                 "memory) and one chunk for the chain (every hop through shared memory); "
                                 "floor = nlevels x t_hop of the path the case's schedule uses",
                          "hw_hop_global_ns": list(HW_HOP_GLOBAL_NS), "hw_hop_smem_cycles": HW_HOP_SMEM_CYCLES,
                          "hw_floor_ms_per_step": [round(sum(d["hw_hop_floor_ms"][0] for d in details.values()), 4),
                                                   round(sum(d["hw_hop_floor_ms"][1] for d in details.values()), 4)],
                          "hw_how": "nlevels x the hardware hop alone (stand-alone probe: relaxed flag hop SM to SM "
                                    "303-464 ns by box; shared-memory hop 196 cycles at the sampled SM clock); "
                                    "per case exec_over_hw_hop_floor gives the range"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_val, 3), "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_step, 4)},
        "gpu_launches": args.steps * len(cases),
        "clocks": clock_info,
        "wall_s_timed": round(t_wall, 3),
        "cases": details,
        "reference_scheme_gpu": ({"ms_per_step": round(sum(ref_scheme.values()), 4),
                                  "gbs": round(total_bytes / (sum(ref_scheme.values()) * 1e-3) / 1e9, 3),
                                  "what": "the reference's warp-per-column push executor scheme (in-degree counters + "
                                          "atomic partial sums), restated with ticket order and bounded waits, "
                                          "same systems, L2 not flushed"} if ref_scheme else None),
    }
    if world == 1 and not args.no_extras and args.scale == 1.0 and not args.cases:
        # the rest of the metric, measured after the headline's timed region:
        # 10k system beside the CPU serial executor, many right-hand sides with
        # mixed precision, the 512-system batch, forward + adjoint
        from sptrsv_gb300 import matgen
        for c in cases:
            c["solver"].close()
        del cases, solvers
        torch.cuda.empty_cache()
        ex_args = argparse.Namespace(**vars(args))
        ex_args.steps = min(args.steps, 10)
        ex_args.rhs_list = [1, 16, 64]
        m1 = matgen.system_1m(seed=2)
        t0 = time.perf_counter()
        line["system_10k"] = measure_system_10k(ex_args, dev)
        line["multi_rhs"] = measure_multi_rhs(ex_args, dev, m=m1)
        line["batch"] = measure_batch(ex_args, dev)
        line["adjoint"] = measure_adjoint(ex_args, dev, m=m1)
        line["extras_wall_s"] = round(time.perf_counter() - t0, 1)
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


# ------------------------------------------------------------------ other workloads
# Each returns a dict; `--workload X` prints it as a line of its own, and the
# default run attaches all four to its line (one GPU, after the timed region
# of the headline workload).
def _timed(fn, reps, flush=None):
    import torch
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def _relerr(x, ref) -> float:
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(float(np.max(np.abs(ref))), 1e-300))


def measure_system_10k(args, dev) -> dict:
    """10k-row Poisson(8) band system, FP64, rhs 1: the serial executor on one host core
    beside the GPU solve (automatic plan), both against the oracle."""
    import torch

    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.system_10k()
    b = m.matvec(np.ones(m.n))
    imp = oracle.ref() or oracle.port()
    deg = imp.analyser(m.row_idx, m.n)
    ts = []
    for _ in range(max(args.steps, 20)):
        t0 = time.perf_counter()
        ref = imp.executor(m.col_ptr, m.row_idx, m.val, deg, m.n, 0, 1, b)
        ts.append(1e3 * (time.perf_counter() - t0))
    cpu_ms = statistics.median(ts)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val, sync_check=False)
    bd = torch.from_numpy(b).to(dev)
    x = s.solve(bd)
    clocks = ClockSampler(dev.index)
    clocks.start()
    time.sleep(0.2)
    # enough repetitions (~0.1 s) for the clock sampler to see the solves
    gpu_ms = _timed(lambda: s.solve(bd, out=x), max(args.steps, 500), flush)
    clk = clocks.stop()
    s.check()
    err = _relerr(x.cpu().numpy(), ref)
    ex = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val, schedule=2, exact=True)
    bit_equal = bool(np.array_equal(ex.solve(bd).cpu().numpy().view(np.uint64), ref.view(np.uint64)))
    ex.close()
    nl = s.info()["nlevels"]
    s.close()
    bp = bytes_pass(m.n, m.nnz)
    return {"workload": "n=10,000 Poisson(8) band 2000, FP64, rhs=1, forward", "n": m.n, "nnz": m.nnz,
            "nlevels": nl, "gpu_ms": round(gpu_ms, 4), "gpu_gbs": round(bp / gpu_ms / 1e6, 3),
            "cpu_serial_ms": round(cpu_ms, 4), "cpu_serial_gbs": round(bp / cpu_ms / 1e6, 3),
            "cpu_kind": "reference" if imp.kind == "ref" else "port", "cpu_cores": 1,
            "speedup_gpu_vs_cpu_serial": round(cpu_ms / gpu_ms, 2), "fwd_err_vs_oracle": err,
            "exact_mode_bit_identical": bit_equal, "l2": "flushed before every GPU solve", "clocks": clk}


def measure_multi_rhs(args, dev, m=None, world=1, rank=0, dist=None) -> dict:
    """n = 1M band system, rhs in {1, 16, 64}, column-major B ~ N(0,1): plain FP64
    vs FP32 storage/solve + FP64-residual refinement, both against the oracle."""
    import torch

    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver, matgen, shard
    if m is None:
        m = matgen.system_1m(seed=2, n=int(round(1_000_000 * args.scale)))
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    out = {}
    clocks = ClockSampler(dev.index)
    clocks.start()
    time.sleep(0.2)
    for rhs in args.rhs_list:
        rng = np.random.default_rng(rhs)
        B = rng.standard_normal((m.n, rhs))
        # the right-hand sides shard over ranks as contiguous column slices;
        # every rank holds the whole triangle and its analysis
        c0, c1 = shard.rhs_columns(rhs, world, rank)
        w = c1 - c0
        t64 = tmix = 0.0
        err64 = errmix = 0.0
        iters = 0
        if w > 0:
            Bl = B[:, c0:c1]
            ref = oracle.port().solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution,
                                      Bl if w > 1 else Bl[:, 0])
            ref = ref.reshape(m.n, w)
            b = torch.from_numpy(np.ascontiguousarray(Bl.T)).to(dev).t()
            s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, sync_check=False,
                               **args.solver_kw)
            x = s.solve(b)
            t64 = _timed(lambda: s.solve(b, out=x), args.steps, flush)
            s.check()
            err64 = _relerr(x.cpu().numpy(), ref)
            s.set_option(7, 1)
            xr, iters, est = s.solve_refine(b)
            s.set_option(7, 0)
            tmix = _timed(lambda: s.solve_refine(b, out=xr, tol=0.0, max_iter=iters), args.steps, flush)
            s.check()
            errmix = _relerr(xr.cpu().numpy(), ref)
            s.close()
        if dist is not None:
            # whole-job time = the slowest rank; errors = the worst slice
            t = torch.tensor([t64, tmix, err64, errmix, iters], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            t64, tmix, err64, errmix = (float(v) for v in t.tolist()[:4])
            iters = int(t[4].item())
        bp = bytes_pass(m.n, m.nnz, rhs)
        out[f"rhs{rhs}"] = {"fp64_ms": round(t64, 4), "mixed_ms": round(tmix, 4), "refine_steps": iters,
                            "speedup_mixed_vs_fp64": round(t64 / tmix, 3), "fp64_fwd_err_vs_oracle": err64,
                            "mixed_fwd_err_vs_oracle": errmix, "fp64_problem_gbs": round(bp / t64 / 1e6, 2),
                            "mixed_problem_gbs": round(bp / tmix / 1e6, 2),
                            "fp64_solves_per_s": round(1e3 / t64, 1)}
    clk = clocks.stop()
    return {"workload": f"n={m.n:,} Poisson(9) band 20k, rhs {'/'.join(map(str, args.rhs_list))}, "
                        "column-major B ~ N(0,1)", "n": m.n, "nnz": m.nnz,
            "cases": out, "l2": "flushed before every solve", "clocks": clk,
            "parallelism": f"rhs columns sharded over {world} rank(s)" if world > 1 else "one GPU"}


def measure_batch(args, dev, world=1, rank=0, dist=None) -> dict:
    """512 independent systems (even lower, odd upper), rhs 4: one batched launch
    sequence (FP32 + FP64 refinement; plain FP64) vs 512 per-system FP64 launches;
    every system's slice against its own oracle solve."""
    import torch

    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver, matgen, shard
    t0 = time.perf_counter()
    systems_all = matgen.batch_uneven(count=args.batch_count, seed=3)
    # independent systems shard over ranks with no exchange (nnz-balanced assignment)
    mine = shard.shard_of([m.nnz for m in systems_all], world, rank)
    systems = [systems_all[k] for k in mine]
    tgen = time.perf_counter() - t0
    rhs = 4
    rng = np.random.default_rng(4)
    bs = [rng.standard_normal((m.n, rhs)) for m in systems]
    ntot = sum(m.n for m in systems)
    nnz = sum(m.nnz for m in systems)
    vals = np.concatenate([m.val for m in systems])
    t0 = time.perf_counter()
    s = SyncFreeSolver(batch=[(m.col_ptr, m.row_idx, m.n, m.substitution) for m in systems], values=vals,
                       sync_check=False, **args.solver_kw)
    tan = time.perf_counter() - t0
    b = torch.from_numpy(np.concatenate(bs)).to(dev)
    tuned = None
    t0 = time.perf_counter()
    if not args.no_tune and not args.solver_kw:
        s.set_option(7, 1)
        tuned = s.tune(b, values=torch.from_numpy(vals).to(dev), reps=2)
        s.set_option(7, 0)
    ttune = time.perf_counter() - t0
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    s.set_option(7, 1)
    xr, iters, est = s.solve_refine(b)
    s.set_option(7, 0)
    x64 = s.solve(b)
    # per-system plain FP64 launches (one handle per system, one launch each)
    hs = [SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, sync_check=False,
                         **args.solver_kw) for m in systems]
    bd = [torch.from_numpy(bb).to(dev) for bb in bs]
    xd = [torch.empty_like(bb) for bb in bd]

    def per_system():
        for h, bb, xx in zip(hs, bd, xd):
            h.solve(bb, out=xx)
    per_system()
    xg = torch.empty_like(xr)
    graph = s.graph(b, xg, kind=1, count=iters)
    graph.replay()
    s.check()
    clocks = ClockSampler(dev.index)
    clocks.start()
    time.sleep(0.2)
    t_mixed = _timed(lambda: s.solve_refine(b, out=xr, tol=0.0, max_iter=iters), args.steps, flush)
    t_graph = _timed(graph.replay, args.steps, flush)
    t_b64 = _timed(lambda: s.solve(b, out=x64), args.steps, flush)
    t_per = _timed(per_system, max(3, args.steps // 3), flush)
    clk = clocks.stop()
    s.check()
    graph_err = float((xg - xr).abs().max() / xr.abs().max())
    graph.close()
    # forward error of every system against its own FP64 oracle solve
    xr_h, x64_h = xr.cpu().numpy(), x64.cpu().numpy()
    xd_h = [xx.cpu().numpy() for xx in xd]
    off = s.offsets
    err_mixed = err64 = err_per = 0.0
    imp = oracle.port()
    for k, m in enumerate(systems):
        ref = imp.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, bs[k])
        err_mixed = max(err_mixed, _relerr(xr_h[off[k]:off[k + 1]], ref))
        err64 = max(err64, _relerr(x64_h[off[k]:off[k + 1]], ref))
        err_per = max(err_per, _relerr(xd_h[k], ref))
    nlevels = s.info()["nlevels"]
    for h in hs:
        h.close()
    s.close()
    if dist is not None:
        # whole-job time = the slowest rank
        t = torch.tensor([t_mixed, t_b64, t_per, t_graph], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_mixed, t_b64, t_per, t_graph = (float(v) for v in t.tolist())
        tot = torch.tensor([ntot, nnz], dtype=torch.float64, device=dev)
        dist.all_reduce(tot)
        ntot, nnz = (int(v) for v in tot.tolist())
        e = torch.tensor([err_mixed, err64, err_per], dtype=torch.float64, device=dev)
        dist.all_reduce(e, op=dist.ReduceOp.MAX)
        err_mixed, err64, err_per = (float(v) for v in e.tolist())
    nsys = len(systems_all)
    return {"workload": f"{nsys} systems (half lower, half upper), n log-uniform 1k-200k, rhs=4",
            "metric": "batched solves/s (FP32+FP64 refinement, one persistent launch per pass)",
            "value": round(nsys / (t_mixed * 1e-3), 2), "unit": "systems/s",
            "systems": nsys, "n_total": ntot, "nnz_total": nnz, "rhs": rhs, "nlevels_batch": nlevels,
            "tuned": tuned, "mixed_batched_ms": round(t_mixed, 3), "refine_steps": iters,
            "mixed_graph_replay_ms": round(t_graph, 3), "graph_vs_direct_rel_diff": graph_err,
            "fp64_batched_ms": round(t_b64, 3), "fp64_batched_solves_per_s": round(nsys / (t_b64 * 1e-3), 2),
            "fp64_per_system_launches_ms": round(t_per, 3),
            "speedup_vs_per_system_fp64": round(t_per / t_mixed, 2),
            "speedup_vs_batched_fp64": round(t_b64 / t_mixed, 3),
            "fwd_err_vs_oracle_mixed": err_mixed, "fwd_err_vs_oracle_fp64_batched": err64,
            "fwd_err_vs_oracle_fp64_per_system": err_per, "checked_systems": len(systems),
            "generate_s": round(tgen, 1), "analyse_s": round(tan, 2), "tune_s": round(ttune, 1),
            "l2": "flushed before every timed call", "clocks": clk,
            "parallelism": f"systems sharded over {world} rank(s), nnz-balanced" if world > 1 else "one GPU"}


def measure_adjoint(args, dev, m=None) -> dict:
    """The 1M band system, rhs 8, FP64, loss = sum(w * x): forward + adjoint with the
    value gradient over the forward time; gradients against the oracle gradient."""
    import torch

    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver, matgen, sparse_triangular_solve
    if m is None:
        m = matgen.system_1m(seed=2)
    rhs = 8
    rng = np.random.default_rng(4)
    Bh = rng.standard_normal((m.n, rhs))
    Wh = rng.standard_normal((m.n, rhs))
    B = torch.from_numpy(Bh).to(dev)
    W = torch.from_numpy(Wh).to(dev)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, sync_check=False, **args.solver_kw)
    val = torch.from_numpy(m.val).to(dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def fwd():
        with torch.no_grad():
            return sparse_triangular_solve(s, val, B)

    def fwd_bwd():
        v = val.detach().requires_grad_(True)
        bb = B.detach().requires_grad_(True)
        x = sparse_triangular_solve(s, v, bb)
        (W * x).sum().backward()
        return x, v.grad, bb.grad
    fwd()
    x, gv, gb = fwd_bwd()
    s.check()
    clocks = ClockSampler(dev.index)
    clocks.start()
    time.sleep(0.2)
    t_f = _timed(fwd, args.steps, flush)
    t_fb = _timed(fwd_bwd, args.steps, flush)
    s.set_option(15, 1)
    fwd_bwd()
    t_fb_fused = _timed(fwd_bwd, args.steps, flush)
    s.set_option(15, 0)
    clk = clocks.stop()
    s.check()
    x_ref = oracle.port().solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, Bh)
    lam_ref, dval_ref = oracle.adjoint_gradient(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, x_ref, Wh)
    errs = {"x": _relerr(x.detach().cpu().numpy(), x_ref), "grad_b": _relerr(gb.cpu().numpy(), lam_ref),
            "grad_values": _relerr(gv.cpu().numpy(), dval_ref)}
    s.close()
    return {"workload": "n=1M Poisson(9) band 20k, rhs=8, FP64, loss=sum(w*x)",
            "metric": "(forward + adjoint with value gradient) / forward time",
            "value": round(t_fb / t_f, 3), "unit": "ratio", "higher_is_better": False,
            "forward_ms": round(t_f, 3), "forward_backward_ms": round(t_fb, 3),
            "forward_backward_fused_in_solve_ms": round(t_fb_fused, 3), "n": m.n, "nnz": m.nnz, "rhs": rhs,
            "err_vs_oracle": errs, "l2": "flushed before every timed call", "clocks": clk}


def _dist_setup(dev, world):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("nccl", device_id=dev)
    return dist


def run_workload(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.workload == "system_10k":
        if rank != 0:
            return 0
        line = measure_system_10k(args, dev)
    elif args.workload == "adjoint":
        if rank != 0:
            return 0
        line = measure_adjoint(args, dev)
    else:
        dist = _dist_setup(dev, world)
        fn = measure_multi_rhs if args.workload == "multi_rhs" else measure_batch
        line = fn(args, dev, world=world, rank=rank, dist=dist)
        if dist is not None:
            dist.destroy_process_group()
            if rank != 0:
                return 0
    line = {"workload_name": args.workload, "n_gpus": world, **line}
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-ref-scheme", action="store_true",
                    help="skip timing the reference's GPU scheme (kernel-level executor) beside the library")
    ap.add_argument("--schedule", type=int, default=None)
    ap.add_argument("--lanes", type=int, default=None)
    ap.add_argument("--chunk", type=int, default=None)
    ap.add_argument("--order-block", type=int, default=None)
    ap.add_argument("--workload", choices=["deep_wide", "system_10k", "multi_rhs", "batch", "adjoint"],
                    default="deep_wide")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload only: skip the 10k, multi-rhs, batch and adjoint measurements "
                         "attached to its line")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--rhs-list", default="1,16,64",
                    help="multi_rhs workload: right-hand-side counts (comma-separated; profiling runs)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="size factor of the deep/wide systems (1.0 = the benchmark sizes; smaller for profiling)")
    ap.add_argument("--cases", default=None,
                    help="comma-separated subset of " + ",".join(CASE_NAMES) + " (profiling runs)")
    ap.add_argument("--opt", action="append", default=[], metavar="KEY=VALUE",
                    help="SyncFreeSolver option (e.g. warp_sync=1, split=32, staged=0); disables the autotuner")
    args = ap.parse_args(argv)
    if args.cases:
        args.cases = [c.strip() for c in args.cases.split(",") if c.strip()]
        bad = [c for c in args.cases if c not in CASE_NAMES]
        if bad:
            ap.error(f"unknown case(s) {bad}")
    if args.warmup < 3:
        args.warmup = 3
    args.rhs_list = [int(v) for v in args.rhs_list.split(",") if v.strip()]
    kw = {}
    for k in ("schedule", "lanes", "chunk", "order_block"):
        v = getattr(args, k)
        if v is not None:
            kw[k] = v
    for o in args.opt:
        k, _, v = o.partition("=")
        if not k or not v:
            ap.error(f"--opt wants KEY=VALUE, got {o!r}")
        kw[k.strip()] = int(v)
    args.solver_kw = kw
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.workload != "deep_wide":
        return run_workload(args, world, rank, local)
    return run_gpu(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
