#!/usr/bin/env python3
"""Benchmark: verified flips/s of the batched uneven Z2 flip-graph search on one GB300.

Workload (the batched uneven search): 65,536 concurrent walks split evenly
over the shapes (2,2,2), (2,2,3), (2,3,4), (3,3,4), (3,4,5), (4,4,4), each
starting from its naive rank n1*n2*n3 scheme, uniform flip-pair proposal
(fast Philox stream), plus transition after 10^5 flips without a rank drop,
expand probability 0.01 (the reference's default).  One step = one launch of
the walk kernel over every walk (`--iterations` steps each, default 10,000 =
the reference's --max-iterations) followed by the exact Brent check of every
walk; only flips of walks whose scheme verifies are counted.

Timing: W warm-up steps, then K timed steps bracketed by a device sync (and a
barrier under torchrun); device time comes from CUDA events recorded by the
library on its launching stream.  The walk records (~600 MB) exceed the
129 MB L2, so no L2 flush is needed between steps.

`e2e` repeats the step through the C ABI with page-locked host records: each
step uploads the records (fg_set_records), runs, and downloads them
(fg_get_records); the copies are inside the timed region.

`--impl reference` times the reference's algorithm on the host CPU cores (the
CPU restatement of its list-mode walk in oracle/, all cores): the reference has
no host walker of its own (its walk operators are __device__-only,
scheme_z2.cuh:40-54).

Keys beside the headline, all measured after the timed region:
  ref_cuda  the reference's own CUDA build (oracle/_ref, compiled from its
            sources) on the same workload: its unmodified randomWalkKernel
            timed with CUDA events, accepted flips counted by a twin kernel
            checked state-for-state against it;
  bitexact  this engine's reference mode (bit-exact trajectories) on the same
            workload; bitexact_by_shape the same for both rings at 16,384 walks
            of 3x3x3 and 4x4x4 beside the reference's build;
  ttr       time to rank 23 on 3x3x3 (1,024 walks) for the fast, bit-exact and
            learned-proposal modes and the reference's CUDA build, 3 seeds;
  ttr_444   time to rank 47 on 4x4x4 (65,536 walks) within a 60 s budget.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPES = [(2, 2, 2), (2, 2, 3), (2, 3, 4), (3, 3, 4), (3, 4, 5), (4, 4, 4)]
# factor word of the Z2 kernels: 32-bit in the fast mode (factors of <= 24 entries,
# every shape here), 64-bit in the list modes
WORD_BYTES = {"fast": 4, "philox": 8, "reference": 8}
DTYPE = {"fast": "u32", "philox": "u64", "reference": "u64"}
METRIC = "verified flips/s"
CONFIG_NAME = "batched uneven Z2 search: 65,536 walks over (2,2,2),(2,2,3),(2,3,4),(3,3,4),(3,4,5),(4,4,4)"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def shape_ranges(walks):
    """Contiguous, even split of the walks over SHAPES: [(shape, first, count)]."""
    out, first = [], 0
    for i, s in enumerate(SHAPES):
        last = (i + 1) * walks // len(SHAPES)
        out.append((s, first, last - first))
        first = last
    return out


def shapes_for(walks):
    sh = np.zeros((walks, 3), np.int32)
    for s, first, count in shape_ranges(walks):
        sh[first:first + count] = s
    return sh


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def smem_peak_gbs():
    """Shared-memory bandwidth of the GPU: 32 banks x 4 B per clock per SM."""
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    mhz = peaks.get("sm_max_mhz", 2070.0)
    sms = 152
    try:
        import ctypes
        cudart = ctypes.CDLL("libcudart.so")
        v = ctypes.c_int()
        if cudart.cudaDeviceGetAttribute(ctypes.byref(v), 16, 0) == 0:  # cudaDevAttrMultiProcessorCount
            sms = v.value
    except OSError:
        pass
    return 128.0 * sms * mhz * 1e6 / 1e9, peaks, sms, mhz


# ------------------------------------------------------------------ CPU side
# The oracle's two walks: "philox" is the reference's list algorithm (FlipSet lists, the
# reference's candidate order and draw sites, scheme_z2.cu:531-641,982-1154) on the
# Philox stream; "fast" is this engine's fast-mode walk (partner counts, canonical pair
# order).  The reference itself has no host walker (its operators are __device__-only).
CPU_WALKS = {"philox": "the reference's list-mode walk (FlipSet lists) on the Philox stream",
             "fast": "the fast-mode walk (partner counts, canonical pair order) on the Philox stream"}


def cpu_walks(walks_per_shape, iterations, plus, seed, threads, rng="philox"):
    """Oracle (CPU restatement) walks over every shape; returns (verified flips, seconds, walks)."""
    from oracle import oracle as O
    jobs = []
    for si, (n1, n2, n3) in enumerate(SHAPES):
        for part in range(threads):
            k = walks_per_shape // threads + (1 if part < walks_per_shape % threads else 0)
            if k:
                jobs.append((n1, n2, n3, k, seed * 1000 + si * 64 + part))
    results = []

    def work(job):
        n1, n2, n3, k, sd = job
        b = O.WalkBatch(k, 64, "z2")
        O.init_naive(b, n1, n2, n3)
        cfg = b.cfg(rng, iterations=iterations, plus_iterations=plus, launches=1, expand_p=0.01, seed=sd)
        O.walk(b, cfg)
        ok = O.validate(b)
        results.append((int(b.accepted[ok].sum()), int(b.accepted.sum())))

    import concurrent.futures as cf
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, jobs))
    dt = time.perf_counter() - t0
    return sum(r[0] for r in results), dt, sum(j[3] for j in jobs)


def cpu_sample(rng, seconds_target, threads, wps):
    """Grows the sample until it is about seconds_target of CPU work (at least a third of it)."""
    iters = 200
    while True:
        v, dt, nw = cpu_walks(wps, iters, 100000, 8, threads, rng)
        if dt >= seconds_target / 3 or iters >= 10_000_000:
            return v, dt, nw, iters
        iters = int(iters * min(50.0, max(2.0, seconds_target / max(dt, 1e-3))))


def cpu_baseline(args, seconds_target=8.0):
    """The oracle on all host cores: the reference's list algorithm (value) and the fast-mode
    walk (fast_mode_port), each a bounded sample of the benchmark's six shapes."""
    threads = os.cpu_count() or 1
    wps = max(threads, 16)
    cpu_walks(wps, 10, 100000, 6, threads)  # loads the oracle library outside the timed samples
    out = {}
    for rng in ("philox", "fast"):
        v, dt, nw, iters = cpu_sample(rng, seconds_target, threads, wps)
        out[rng] = {"value": v / dt, "unit": METRIC, "walk": CPU_WALKS[rng],
                    "sample": f"{nw} walks ({wps} per shape) x {iters} steps, {threads} host threads, {dt:.1f} s"}
    lst = out["philox"]
    return {"value": lst["value"], "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{lst['walk']}: {lst['sample']}", "fast_mode_port": out["fast"]}


def reference_arm(args):
    """The reference's algorithm on the host cores: the oracle's restatement of its list-mode
    walk (FlipSet lists, its candidate order and draw sites) on the Philox stream, all host
    threads, over the benchmark's six shapes.  Each step is a bounded sample: --ref-walks-per-shape
    walks of each shape (at least one per thread) x --ref-iterations steps."""
    ws, rank = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    wps = max(threads, args.ref_walks_per_shape)
    iters = args.ref_iterations
    for _ in range(args.warmup):
        cpu_walks(wps, max(10, iters // 10), 100000, 3, threads)
    tot_v, tot_t = 0, 0.0
    nw = 0
    for k in range(args.steps):
        v, dt, nw = cpu_walks(wps, iters, 100000, 100 + k, threads)
        tot_v += v
        tot_t += dt
    value = tot_v / tot_t
    sample = (f"{nw} walks ({wps} per shape of the six) x {iters} steps per step, {CPU_WALKS['philox']}, "
              f"{threads} host threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (naive starting schemes)",
            "config": {"workload": CONFIG_NAME, "walks_sampled": nw, "walks_per_shape": wps,
                       "iterations_per_step": iters, "plus_iterations": 100000, "expand_p": 0.01,
                       "walk": "reference list algorithm (oracle restatement), Philox stream",
                       "note": "a bounded CPU sample of the GPU workload (65,536 walks x 10,000 steps does not fit "
                               "a CPU step); flips/s is per walk-step independent of the walk count"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ reference CUDA build
def ref_harness_path(ring):
    import platform
    p = os.path.join(ROOT, "oracle", "_ref", f"{ring}-{platform.machine()}", "ref_harness")
    return p if os.path.exists(p) else None


def run_ref_harness(ring, argv, timeout):
    """One run of the reference's own CUDA build (oracle/_ref, compiled from its sources by
    oracle/build_ref.sh) outside every timed region; returns its JSON line or a reason."""
    exe = ref_harness_path(ring)
    if exe is None:
        return {"unavailable": f"no reference build for {ring} (oracle/_ref/{ring}-<machine>/ref_harness)"}
    try:
        r = subprocess.run([exe] + [str(a) for a in argv], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                           text=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return {"unavailable": f"ref_harness {argv[0]} exceeded {timeout} s"}
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"unavailable": f"ref_harness {argv[0]} rc={r.returncode}: {r.stderr.strip()[-200:]}"}
    return json.loads(lines[-1])


def ref_cuda_baseline(args, walks, iterations, ours_value):
    """The reference's unmodified randomWalkKernel (flip_graph.cu:520-573, Z2 build) on the
    same six-shape workload, its accepted flips counted exactly by a counting twin run on a
    copy of its state and checked equal state for state; plus its time to rank 23 on 3x3x3."""
    shapes = [f"{a}x{b}x{c}" for a, b, c in SHAPES]
    t = run_ref_harness("z2", ["time", walks, iterations, args.ref_cuda_launches, args.seed, args.plus_iterations]
                        + shapes, timeout=600)
    out = {"workload": f"{CONFIG_NAME}; {iterations} steps per launch, resize off, expand 0.01, plus after "
                       f"{args.plus_iterations}", "kernel": "randomWalkKernel (unmodified, Z2 build, block 32)"}
    if "unavailable" in t:
        out["unavailable"] = t["unavailable"]
        return out
    out.update({"value": t["verified_flips_per_s"], "unit": METRIC, "ms_per_launch": t["ms_per_launch"],
                "launches": t["launches"], "accepted_flips": t["accepted_flips"],
                "verified_flips": t["verified_flips"], "twin_mismatches": t["twin_mismatches"],
                "valid_walks": t["valid_walks"], "best_ranks": t["best_ranks"],
                "ours_over_reference": ours_value / t["verified_flips_per_s"] if t["verified_flips_per_s"] else None})
    return out


# ------------------------------------------------------------------ time to target rank
def ttr_one(fg, mode, shape, walks, target, plus, iters, seconds, seed, net=None, candidates=8, min_entropy=0.05):
    """Wall time from engine creation until a verified best scheme reaches `target` (Z2, naive
    start, plus after `plus` flips without a rank drop, flip limit 10^7 per walk, expand 0.01),
    or the best rank after `seconds`."""
    n1, n2, n3 = shape
    cap = n1 * n2 * n3
    t0 = time.perf_counter()
    eng = fg.Engine(walks, cap, "z2", mode, seed, iters, plus, 0.01, 0.0, 0, 0)
    if mode == "learned":
        eng.set_proposal(net, candidates=candidates, temperature=1.0, min_entropy=min_entropy)
    eng.init_naive(n1, n2, n3)
    reached, launches, best, flips = False, 0, cap, 0
    while launches * iters < 10_000_000 and time.perf_counter() - t0 < seconds:
        st = eng.run(1)
        launches += 1
        flips += st["verified_flips"]
        best = min(best, st["min_best_rank"])
        if st["min_best_rank"] <= target:
            c = eng.counters()
            w = int(np.argmin(c["best_rank"]))
            reached = bool(eng.validate(best=True)[w])
            if reached:
                break
    dt = time.perf_counter() - t0
    eng.close()
    return {"mode": mode, "seed": seed, "reached": reached, "seconds": dt, "launches": launches,
            "steps_per_walk": launches * iters, "best_rank": int(best), "verified_flips": int(flips)}


def ttr_summary(runs):
    ok = [r["seconds"] for r in runs if r["reached"]]
    return {"reached": f"{len(ok)}/{len(runs)}", "median_seconds": statistics.median(ok) if ok else None,
            "median_steps_per_walk": statistics.median([r["steps_per_walk"] for r in runs if r["reached"]]) if ok else None,
            "runs": runs}


def reduce_over_ranks(seconds, units, dist=None):
    """Whole-job figures of the replicas: the slowest rank's time and the units of all ranks
    (one gloo all-reduce each; the walks themselves exchange nothing)."""
    if not dist:
        return seconds, float(units)
    import torch
    t = torch.tensor([seconds], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64)
    dist.all_reduce(u)
    return float(t[0]), float(u[0])


# ------------------------------------------------------------------ GPU side
def gpu_arm(args):
    ws, rank = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    device = int(os.environ.get("LOCAL_RANK", "0"))
    import flipgraphgpu_gb300 as fg
    walks, cap, iters = args.walks, 64, args.iterations
    seed = args.seed + rank
    eng = fg.Engine(walks, cap, "z2", args.mode, seed, iters, args.plus_iterations, 0.01, 0.0, device,
                    args.walks_per_block)
    if args.fast_split is not None:
        eng.set_fast_split(args.fast_split)
    if args.fast_kernel is not None:
        eng.set_fast_kernel(args.fast_kernel, args.lanes)
    shapes = shapes_for(walks)
    eng.init_naive_shapes(shapes)
    kernels = None
    if args.autotune > 0:  # per-segment kernel choice, trajectories unchanged
        names = {0: "thread", 1: "group", 2: "warp"}
        kernels = [f"{names.get(k, 'auto')}{l if k == 1 else ''}{f'/{w}w' if k == 0 else ''}"
                   for k, l, w in eng.autotune(args.autotune)]
    for _ in range(args.warmup):
        eng.run(1)

    def barrier():
        if dist:
            dist.barrier()

    clocks = ClockSampler(device)
    # ---- device-resident timed region
    barrier()
    clocks.start()
    wall0 = time.perf_counter()
    kern_ms = ver_ms = 0.0
    flips = vflips = 0
    algo_bytes = 0.0
    per_shape = {s: [0, 0] for s in SHAPES}
    m_prev = eng.counters()["m"]
    for _ in range(args.steps):
        st = eng.run(1)
        kern_ms += st["kernel_ms"]
        ver_ms += st["verify_ms"]
        flips += st["flips"]
        vflips += st["verified_flips"]
        c = eng.counters()
        mavg = 0.5 * (c["m"] + m_prev)
        m_prev = c["m"]
        f = c["flips"].astype(np.float64)
        algo_bytes += float(np.sum(f * (2 * mavg + 4) * WORD_BYTES[args.mode]))
        for s, first, count in shape_ranges(walks):
            sel = slice(first, first + count)
            per_shape[s][0] += int(c["flips"][sel][c["valid"][sel]].sum())
    wall = time.perf_counter() - wall0
    barrier()
    clk = clocks.stop()
    dev_s, vflips_all = reduce_over_ranks((kern_ms + ver_ms) / 1000.0, vflips, dist)
    value = vflips_all / dev_s
    best = eng.counters()
    best_rank = {f"{a}x{b}x{c}": int(best["best_rank"][f:f + n].min()) for (a, b, c), f, n in shape_ranges(walks)}
    shape_rate = {f"{a}x{b}x{c}": per_shape[(a, b, c)][0] / dev_s for (a, b, c) in SHAPES}

    # ---- end to end through the C ABI with page-locked host records
    rec = fg.Records(walks, cap, "z2", pinned=True, lists=args.mode != "fast")  # the fast mode keeps no lists
    eng.records(into=rec)
    h2d = d2h = rec.nbytes()
    barrier()
    e0 = time.perf_counter()
    ev = 0
    for _ in range(args.e2e_steps):
        eng.set_records(rec)
        st = eng.run(1)
        eng.records(into=rec)
        ev += st["verified_flips"]
    e_wall = time.perf_counter() - e0
    barrier()
    e2e_value = ev * ws / e_wall

    smem_peak, peaks, sms, mhz = smem_peak_gbs()
    achieved = algo_bytes / (kern_ms / 1000.0) / 1e9
    traffic, issue = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "bench_traffic.json")) as f:
            prof = json.load(f)
        traffic = prof["dram_bytes_per_step"]
        issue = {"bound": "issue", "frac": prof["issue_active_pct"] / 100.0, "kernel": prof["issue_kernel"],
                 "source": prof["issue_source"]}
    except (OSError, KeyError, ValueError):
        pass
    eng.close()
    if rank == 0:
        cpu = cpu_baseline(args) if (ws == 1 and not args.no_cpu) else None
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dev_s / args.steps, "wall_ms_per_step": 1000 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.mode],
            "data": "synthetic (naive starting schemes)",
            "config": {"workload": CONFIG_NAME, "walks": walks, "iterations_per_step": iters,
                       "plus_iterations": args.plus_iterations, "expand_p": 0.01, "mode": args.mode,
                       "walks_per_block": args.walks_per_block, "l2": "records larger than L2 (no flush)",
                       "parallelism": f"replicas x{ws}", "kernels_by_shape": kernels,
                       "launch": "per step: one CUDA graph of the shape segments' kernels, then the exact check"},
            "flips_per_s_by_shape": shape_rate, "best_rank_by_shape": best_rank,
            "flips": flips, "verified_flips": vflips,
            "kernel_ms_per_step": kern_ms / args.steps, "verify_ms_per_step": ver_ms / args.steps,
            "gpu_launches": args.steps * (1 + (len(SHAPES) if args.mode == "fast" else 1)),
            "roofline": {"bound": "smem", "achieved": achieved, "peak": smem_peak, "unit": "GB/s",
                         "frac": achieved / smem_peak, "traffic": traffic,
                         "traffic_note": "DRAM bytes of one step's walk launches (ncu capture, profiles/bench_launch_list.md)",
                         "peak_source": f"derived: 128 B/clk/SM x {sms} SMs x {mhz:.0f} MHz (sm_max_mhz, MEASURED_PEAKS.json)",
                         "algorithmic_bytes": f"per accepted flip (2m+4) x {WORD_BYTES[args.mode]} B of shared-memory traffic",
                         "binding": issue},
            "clocks": clk,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": args.e2e_steps},
            "cpu_baseline": cpu,
        }
        if ws == 1 and not args.no_extras:
            line.update(extras(fg, args, value))
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def bitexact_leg(fg, args, walks, iterations):
    """This engine's reference mode (bit-exact with the reference's kernel: its cuRAND XORWOW
    stream, FlipSet lists and draw order) on the benchmark's six-shape workload."""
    eng = fg.Engine(walks, 64, "z2", "reference", args.seed, iterations, args.plus_iterations, 0.01, 0.0, 0, 0)
    eng.init_naive_shapes(shapes_for(walks))
    eng.run(1)
    v, ms = 0, 0.0
    for _ in range(args.ref_cuda_launches):
        st = eng.run(1)
        v += st["verified_flips"]
        ms += st["kernel_ms"] + st["verify_ms"]
    eng.close()
    return {"value": v / (ms / 1000.0), "unit": METRIC, "mode": "reference (bit-exact, XORWOW, FlipSet lists)",
            "launches": args.ref_cuda_launches, "iterations_per_launch": iterations, "walks": walks,
            "kernel": "thread per walk, static choice (6 warps per block: several Z2 segments)"}


def bitexact_by_shape(fg, args, walks=16384, iterations=200):
    """This engine's bit-exact reference mode beside the reference's own CUDA build, both rings,
    16,384 walks of one shape (3x3x3 and 4x4x4), 200 steps per launch, plus after 10^5."""
    rows = []
    for ring in ("zt", "z2"):
        for n1, n2, n3 in ((3, 3, 3), (4, 4, 4)):
            eng = fg.Engine(walks, n1 * n2 * n3, ring, "reference", args.seed, iterations, 100000, 0.01, 0.0, 0, 0)
            eng.init_naive(n1, n2, n3)
            eng.run(1)
            v, ms = 0, 0.0
            for _ in range(2):
                st = eng.run(1)
                v += st["verified_flips"]
                ms += st["kernel_ms"] + st["verify_ms"]
            eng.close()
            ours = v / (ms / 1000)
            ref = run_ref_harness(ring, ["time", walks, iterations, 2, args.seed, 100000, f"{n1}x{n2}x{n3}"],
                                  timeout=600)
            row = {"ring": ring.upper(), "shape": f"{n1}x{n2}x{n3}", "walks": walks, "iterations_per_launch": iterations,
                   "ours": ours}
            if "unavailable" in ref:
                row["ref_cuda"] = ref
            else:
                row.update({"ref_cuda": ref["verified_flips_per_s"], "twin_mismatches": ref["twin_mismatches"],
                            "ours_over_reference_cuda": ours / ref["verified_flips_per_s"]})
            rows.append(row)
    return {"unit": METRIC, "mode": "reference (bit-exact)", "rows": rows}


def extras(fg, args, value):
    """Keys beside the headline, each outside the timed region: the reference's own CUDA build
    on the same workload (ref_cuda), this engine's bit-exact mode there (bitexact), time to rank
    23 on 3x3x3 per mode (ttr), time to rank 47 on 4x4x4 (ttr_444) and the additions reducer
    beside the reference's (reducer)."""
    log = lambda msg: print(f"[bench] {msg}", file=sys.stderr, flush=True)  # noqa: E731
    out = {}
    t = time.perf_counter()
    ref = ref_cuda_baseline(args, args.walks, args.iterations, value)
    be = bitexact_leg(fg, args, args.walks, args.iterations)
    if "value" in ref:
        be["over_reference_cuda"] = be["value"] / ref["value"]
    out["ref_cuda"], out["bitexact"] = ref, be
    out["bitexact_by_shape"] = bitexact_by_shape(fg, args)
    log(f"ref_cuda and bitexact legs {time.perf_counter() - t:.1f} s")
    # time to rank 23 on 3x3x3 (1,024 walks, plus after 50,000, flip limit 10^7)
    t = time.perf_counter()
    shape, target, walks = (3, 3, 3), 23, 1024
    with fg.Engine(32, 27, "z2", "fast", 1, 10, 50000) as warm:  # CUDA context and module load
        warm.init_naive(*shape)
        warm.run(1)
    ttr = {"workload": "time to rank 23, 3x3x3 Z2, 1,024 walks from the naive scheme, plus after 50,000 flips, "
                       "flip limit 10^7 per walk, wall time from engine creation, every scheme verified exactly"}
    for mode, iters in (("fast", 1000), ("reference", 1000)):
        ttr[mode] = ttr_summary([ttr_one(fg, mode, shape, walks, target, 50000, iters, 60.0, sd)
                                 for sd in args.ttr_seeds])
    net, info = train_proposal(fg, args)
    ttr["learned"] = ttr_summary([ttr_one(fg, "learned", shape, walks, target, 50000, 200, 60.0, sd, net=net,
                                          candidates=args.learned_candidates) for sd in args.ttr_seeds])
    ttr["learned"]["training"] = info
    net.close()
    refruns = []
    for sd in args.ttr_seeds:
        r = run_ref_harness("z2", ["ttr", 3, 3, 3, walks, 1000, 50000, sd, target, 60], timeout=120)
        if "unavailable" not in r:
            r = {"mode": "reference CUDA build", "seed": sd, **r, "reached": bool(r.get("reached"))}
        refruns.append(r)
    ttr["reference_cuda"] = (ttr_summary(refruns) if all("unavailable" not in r for r in refruns)
                             else {"unavailable": refruns[0].get("unavailable")})
    fast, lrn = ttr["fast"]["median_seconds"], ttr["learned"]["median_seconds"]
    ttr["learned_over_uniform_time"] = lrn / fast if (fast and lrn) else None
    out["ttr"] = ttr
    log(f"ttr legs {time.perf_counter() - t:.1f} s")
    # time to rank 47 on 4x4x4 (65,536 walks, plus after 10^5, within a 60 s budget)
    t = time.perf_counter()
    r = ttr_one(fg, "fast", (4, 4, 4), 65536, 47, 100000, 5000, args.ttr444_seconds, args.seed)
    out["ttr_444"] = {"workload": f"time to rank 47, 4x4x4 Z2, 65,536 walks, plus after 100,000 flips, "
                                  f"{args.ttr444_seconds:.0f} s budget", **r}
    log(f"ttr_444 leg {time.perf_counter() - t:.1f} s")
    t = time.perf_counter()
    out["reducer"] = reducer_leg(fg, args)
    out["minimizer"] = minimizer_leg(fg, args)
    log(f"reducer and minimizer legs {time.perf_counter() - t:.1f} s")
    return out


REDUCER_SCHEME = os.path.join(ROOT, "tests", "golden", "scheme_444_z2_r47.txt")


def read_reducer_scheme():
    """The committed 4x4x4 Z2 scheme of rank 47 as (n, m, coef [1][3][m][64] int8)."""
    tok = [int(x) for x in open(REDUCER_SCHEME).read().split()]
    n, m = tok[:3], tok[3]
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    coef = np.zeros((1, 3, m, 64), np.int8)
    p = 4
    for c in range(3):
        for t in range(m):
            coef[0, c, t, :nn[c]] = tok[p:p + nn[c]]
            p += nn[c]
    return n, m, coef


def searched_scheme_444(fg, path, seed=3):
    """A 4x4x4 Z2 scheme as the minimizer meets them: the current scheme of the lowest-rank walk
    (with at least one equal-factor pair, so that flips exist) after four launches of 5,000
    fast-mode steps over 4,096 walks; written to PATH in the reference's text layout.
    Returns (n, m, factor bitmasks [3][m])."""
    with fg.Engine(4096, 64, "z2", "fast", seed, 5000, 100000, 0.01, 0.0) as eng:
        eng.init_naive(4, 4, 4)
        eng.run(4)
        rec = eng.records()
    n = [4, 4, 4]
    order = np.argsort(rec.m, kind="stable")
    for w in order:
        m = int(rec.m[w])
        fac = rec.fac[w, :, :m]
        if any(len(set(fac[c].tolist())) < m for c in range(3)):
            break
    nn = [16, 16, 16]
    with open(path, "w") as f:
        f.write(f"{n[0]} {n[1]} {n[2]} {m}\n")
        for c in range(3):
            for t in range(m):
                f.write(" ".join(str((int(fac[c, t]) >> j) & 1) for j in range(nn[c])) + "\n")
    return n, m, fac.copy()


def minimizer_leg(fg, args, count=4096, iterations=2000, launches=2, seed=3):
    """The complexity minimizer (minimizeKernel, complexity_minimizer.cu:173-214) on COUNT copies
    of one searched 4x4x4 Z2 scheme: this engine's bit-exact minimizer (the reference's cuRAND
    stream and FlipSet lists) beside the reference's own CUDA build, LAUNCHES launches of
    ITERATIONS flips from the same start; every walk's best complexity is compared."""
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "scheme_444.txt")
        n, m, fac = searched_scheme_444(fg, path, seed)
        nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
        rec = fg.Records(count, m, "z2")
        rec.n[:] = n
        rec.m[:] = m
        rec.fac[:] = fac[None]
        rec.best_fac[:] = rec.fac
        rec.best_rank[:] = m
        rec.best_m[:] = m
        c0 = int(sum(bin(int(x)).count("1") for x in fac.ravel())) - 2 * m - nn[2]
        with fg.Engine(32, m, "z2", "reference", seed, 10, 10**9, 0.0, 0.0) as warm:  # module load, attributes
            warm.set_records(_first_walks(fg, rec, 32))
            warm.rebuild_lists()
            warm.minimize(np.full(32, c0, np.int32))
        eng = fg.Engine(count, m, "z2", "reference", seed, iterations, 10**9, 0.0, 0.0)
        eng.set_records(rec)
        eng.rebuild_lists()
        bc = np.full(count, c0, np.int32)
        flips, t = 0, time.perf_counter()
        for _ in range(launches):
            bc = eng.minimize(bc)
            flips += int(eng.counters()["flips"].sum())
        dt = time.perf_counter() - t
        ok = eng.validate(best=True)
        eng.close()
        out = {"workload": f"complexity minimizer, {count} copies of one searched 4x4x4 Z2 scheme of rank {m} "
                           f"(complexity {c0}), {launches} launches of {iterations} flips, seed {seed}",
               "unit": "verified flips/s", "ours": flips / dt if dt > 0 else None, "ours_seconds": dt,
               "flips": flips, "best_complexity": int(bc.min()), "best_schemes_exact": bool(ok.all()),
               "kernel": "bit-exact list-mode minimizer (the reference's stream and pair order), one warp per walk"}
        per = os.path.join(tmp, "ref_minimizer.txt")
        ref = run_ref_harness("z2", ["minimize_time", path, count, iterations, seed, launches, per], timeout=600)
        if "unavailable" in ref:
            out["ref_cuda"] = ref
            return out
        ref_bc = np.array([int(x) for x in open(per).read().split()], np.int64)
    same = len(ref_bc) == count and bool(np.array_equal(ref_bc, bc))
    ref_s = ref["ms_per_launch"] * launches / 1000.0
    # identical best complexities: the reference's build made the same flips
    out.update({"ref_cuda": flips / ref_s if same and ref_s > 0 else None, "ref_cuda_seconds": ref_s,
                "ref_kernel": "minimizeKernel (unmodified, Z2 build, block 32)",
                "ours_over_reference_cuda": ref_s / dt if same and dt > 0 else None,
                "identical_to_reference": same})
    return out


def _first_walks(fg, rec, k):
    """Records of the first k walks of rec."""
    sub = fg.Records(k, rec.cap, rec.ring)
    for name, _ in fg.Records.FIELDS:
        a, b = getattr(rec, name, None), getattr(sub, name, None)
        if a is not None and b is not None:
            b[...] = a[:k]
    return sub


def reducer_leg(fg, args, count=4096, seed=3):
    """The additions reducer (runReducersKernel, scheme_additions_reducer.cu:494-540) on a 4x4x4
    Z2 scheme of rank 47 (found by this engine's search, a committed fixture): COUNT reducers,
    one launch each side, this engine beside the reference's own CUDA build with the same
    seed; both are bit-exact, so every reducer's U, V and W addition counts and modes are
    compared too."""
    n, m, coef = read_reducer_scheme()
    warm = fg.Reducer(n, m, coef, count=32, schemes=1, seed=seed, threads=512)  # module load, attributes
    warm.run(want_vars=False)
    warm.close()
    red = fg.Reducer(n, m, coef, count=count, schemes=1, seed=seed, threads=512)
    t = time.perf_counter()
    got = red.run(want_vars=False)  # synchronous: launch, then the counts copied back
    dt = time.perf_counter() - t
    red.close()
    out = {"workload": f"additions reducer, {count} reducers on one 4x4x4 Z2 scheme of rank 47, seed {seed}, "
                       "independent (no flips)",
           "unit": "reducer runs/s", "ours": count / dt, "ours_seconds": dt,
           "best_additions": int(got["additions"].sum(axis=1).min()),
           "kernel": "one block of 512 threads per reducer (pair tables in shared memory)"}
    with tempfile.TemporaryDirectory() as tmp:
        per = os.path.join(tmp, "ref_reducers.txt")
        ref = run_ref_harness("zt", ["reduce_time", REDUCER_SCHEME, count, seed, 1, per], timeout=600)
        if "unavailable" in ref:
            out["ref_cuda"] = ref
            return out
        rows = [ln.split() for ln in open(per)]
    same = len(rows) == count and all(
        [int(x) for x in rows[r][:3]] == [int(got["additions"][r, c]) for c in range(3)] and
        rows[r][3:] == [fg.mode_name(got["mode"][r, c], got["scale"][r, c]) for c in range(3)]
        for r in range(count))
    out.update({"ref_cuda": ref["runs_per_s"], "ref_cuda_seconds": ref["ms_per_launch"] / 1000.0,
                "ref_kernel": "runReducersKernel (unmodified, one thread per reducer, block 32)",
                "ours_over_reference_cuda": out["ours"] / ref["runs_per_s"],
                "identical_to_reference": bool(same)})
    return out


def train_proposal(fg, args):
    """Trains the flip-proposal network on records of plain walks of 3x3x3 (the time-to-rank
    workload's shape); returns (net, summary)."""
    t0 = time.perf_counter()
    feats, labels, total, launches = [], [], 0, 0
    with fg.Engine(16384, 27, "z2", "learned", args.seed, 2000, 50000, 0.01, 0.0) as eng:
        eng.init_naive(3, 3, 3)
        while total < args.ttr_learned_records and launches < 64:
            f, y = eng.collect_records(every=args.learned_every, horizon=args.learned_horizon, launches=2,
                                       capacity=1 << 22)
            feats.append(f)
            labels.append(y)
            total += len(y)
            launches += 2
    f = np.concatenate(feats)[:args.ttr_learned_records]
    y = np.concatenate(labels)[:args.ttr_learned_records]
    t1 = time.perf_counter()
    net = fg.Mlp(seed=args.seed)
    loss = net.train(f, y, batch=8192, epochs=args.learned_epochs, lr=1e-3, seed=args.seed)
    return net, {"records": int(len(y)), "positive_fraction": float(y.mean()) if len(y) else None,
                 "collect_seconds": t1 - t0, "train_seconds": time.perf_counter() - t1, "final_loss": loss,
                 "candidates": args.learned_candidates}


def ttr_arm(args):
    """Time to target rank over Z2 from the naive scheme: --ttr-walks walks of --ttr-shape, plus
    transition after --ttr-plus flips without a rank drop, flip limit 10^7 per walk, stop when a
    verified best scheme reaches --ttr-target.  Launches of --ttr-iterations steps; wall time from
    engine creation.  Prints one JSON line per mode and seed."""
    import flipgraphgpu_gb300 as fg
    shape = tuple(int(x) for x in args.ttr_shape.split("x"))
    with fg.Engine(32, shape[0] * shape[1] * shape[2], "z2", "fast", args.seed, 10, args.ttr_plus) as warm:
        warm.init_naive(*shape)  # CUDA context and module load
        warm.run(1)
    for mode in args.ttr_modes.split(","):
        for sd in args.ttr_seeds:
            r = ttr_one(fg, mode, shape, args.ttr_walks, args.ttr_target, args.ttr_plus, args.ttr_iterations,
                        args.ttr_seconds, sd)
            print(json.dumps({"workload": f"time to rank {args.ttr_target}, {args.ttr_shape} Z2, "
                                          f"{args.ttr_walks} walks", "plus_iterations": args.ttr_plus, **r}))
    return 0


def learned_arm(args):
    """Learned flip proposal against the uniform one on the same GPU.

    1. Records: plain (uniform-proposal) walks from the naive schemes of (3,3,3), (3,4,5) and
       (4,4,4) log every --learned-every-th accepted flip with label "rank dropped within the next
       --learned-horizon flips" (16 and 1000 by default), until --learned-records records exist.
    2. Training: the 192-256-256-1 bf16 MLP on the tensor cores (Adam, --learned-epochs).
    3. Held-out AUC of the scores (a uniform proposal scores 0.5).
    4. Search: for (4,4,4) and (3,4,5), --learned-walks walks each from the naive scheme for
       --learned-seconds seconds with the uniform proposal (fast mode) and with the learned one
       (--learned-candidates candidates per step); flips/s and best verified rank.
    5. Time to rank 23 on (3,3,3) (1,024 walks) with each proposal.
    One JSON line per item."""
    import flipgraphgpu_gb300 as fg
    t0 = time.perf_counter()
    shapes = [(3, 3, 3), (3, 4, 5), (4, 4, 4)]
    per = 16384
    sh = np.array([shapes[w // per] for w in range(per * len(shapes))], np.int32)
    feats, labels = [], []
    total, launches = 0, 0
    with fg.Engine(len(sh), 64, "z2", "learned", args.seed, 2000, 50000, 0.01, 0.0) as eng:
        eng.init_naive_shapes(sh)
        while total < args.learned_records and launches < 64:
            f, y = eng.collect_records(every=args.learned_every, horizon=args.learned_horizon, launches=2,
                                       capacity=1 << 23)
            feats.append(f)
            labels.append(y)
            total += len(y)
            launches += 2
    f = np.concatenate(feats)[:args.learned_records]
    y = np.concatenate(labels)[:args.learned_records]
    t_collect = time.perf_counter() - t0
    perm = np.random.default_rng(args.seed).permutation(len(y))
    f, y = f[perm], y[perm]
    split = int(len(y) * 0.95)
    net = fg.Mlp(seed=args.seed)
    t1 = time.perf_counter()
    loss = net.train(f[:split], y[:split], batch=8192, epochs=args.learned_epochs, lr=1e-3, seed=args.seed)
    t_train = time.perf_counter() - t1
    s = net.score(f[split:])
    order = np.argsort(s, kind="stable")
    ranks = np.empty(len(s))
    ranks[order] = np.arange(len(s))
    pos = y[split:] > 0
    auc = float((ranks[pos].mean() - (pos.sum() - 1) / 2) / max((~pos).sum(), 1))
    print(json.dumps({"workload": "learned proposal: records and training", "records": int(len(y)),
                      "horizon": args.learned_horizon, "every": args.learned_every,
                      "positive_fraction": float(y.mean()), "collect_seconds": t_collect, "train_seconds": t_train,
                      "epochs": args.learned_epochs, "final_loss": loss, "heldout_auc": auc}))
    sys.stdout.flush()

    def search(shape, mode, walks, seconds, iters, target=None):
        n1, n2, n3 = shape
        eng = fg.Engine(walks, n1 * n2 * n3, "z2", mode, args.seed, iters, 50000, 0.01, 0.0)
        if mode == "learned":
            eng.set_proposal(net, candidates=args.learned_candidates, temperature=1.0, min_entropy=0.05)
        eng.init_naive(n1, n2, n3)
        t = time.perf_counter()
        flips, kernel_ms, best, reached, launches = 0, 0.0, n1 * n2 * n3, None, 0
        while time.perf_counter() - t < seconds:
            st = eng.run(1)
            launches += 1
            flips += st["verified_flips"]
            kernel_ms += st["kernel_ms"] + st["verify_ms"]
            best = min(best, st["min_best_rank"])
            if target is not None and best <= target:
                c = eng.counters()
                w = int(np.argmin(c["best_rank"]))
                if eng.validate(best=True)[w]:
                    reached = time.perf_counter() - t
                    break
        wall = time.perf_counter() - t
        eng.close()
        return {"flips_per_s": flips / max(kernel_ms / 1000, 1e-9), "best_rank": int(best), "seconds": wall,
                "reached_seconds": reached, "launches": launches, "steps_per_walk": launches * iters}

    for shape in ((4, 4, 4), (3, 4, 5)):
        for mode in ("fast", "learned"):
            iters = 1000 if mode == "fast" else 200
            r = search(shape, mode, args.learned_walks, args.learned_seconds, iters)
            print(json.dumps({"workload": f"search {shape[0]}x{shape[1]}x{shape[2]} Z2, {args.learned_walks} walks, "
                                          f"{args.learned_seconds:.0f} s", "proposal": "uniform" if mode == "fast" else
                              f"learned ({args.learned_candidates} candidates)", **r}))
            sys.stdout.flush()
    for mode in ("fast", "learned"):
        r = search((3, 3, 3), mode, 1024, 60.0, 200, target=23)
        print(json.dumps({"workload": "time to rank 23, 3x3x3 Z2, 1024 walks",
                          "proposal": "uniform" if mode == "fast" else f"learned ({args.learned_candidates} candidates)",
                          **r}))
        sys.stdout.flush()
    net.close()
    return 0


def post_arm(args):
    """Post-search workload on --post-schemes Z2 schemes of 4x4x4.

    1. Search (config 1's method): 65,536 fast-mode walks of 4x4x4 from the naive scheme for
       --post-search-seconds; the --post-schemes walks with the lowest verified best rank are kept
       (ranks 47-50 typically).
    2. Complexity minimizer: rank-preserving flip walks (fast mode, one thread per walk) on those
       schemes, --post-launches launches of --post-iterations steps; flips/s and complexities.
    3. Additions reducer: --post-reducers reducers per scheme on the minimized schemes, one GPU
       launch per rank group; reducer runs/s and addition counts.
    The addition counts are the reference's for the same scheme and seed (tests/test_gpu_reducer.py
    checks 32 reducers on the rank-47 scheme of tests/golden against the reference kernel)."""
    import flipgraphgpu_gb300 as fg
    log = lambda msg: print(f"[post] {msg}", file=sys.stderr, flush=True)  # noqa: E731
    n, cap, S = (4, 4, 4), 64, args.post_schemes
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    t = time.perf_counter()
    with fg.Engine(65536, cap, "z2", "fast", args.seed, 5000, 100000, 0.01, 0.0) as search:
        search.init_naive(*n)
        while time.perf_counter() - t < args.post_search_seconds:
            search.run(1)
        full = search.records()
        ok = search.validate(best=True)
    t_search = time.perf_counter() - t
    order = np.lexsort((np.arange(len(ok)), full.best_m + 1000 * (~ok)))[:S]
    ranks = full.best_m[order]
    log(f"search {t_search:.1f} s; ranks kept {np.unique(ranks, return_counts=True)}")
    rec = fg.Records(S, cap, "z2")
    rec.n[:] = n
    rec.m[:] = ranks
    rec.fac[:] = full.best_fac[order]
    rec.best_fac[:] = rec.fac
    rec.best_rank[:] = ranks
    rec.best_m[:] = ranks
    c0 = np.array([sum(bin(int(x)).count("1") for x in rec.fac[w, :, :ranks[w]].ravel()) for w in range(S)],
                  np.int64) - 2 * ranks - nn[2]
    # fast mode: the minimizer's flips with the fast walk's stream and pair order, one thread per walk
    eng = fg.Engine(S, cap, "z2", "fast", args.seed, args.post_iterations, 10**9, 0.0, 0.0)
    eng.set_records(rec)
    bc = c0.astype(np.int32)
    bc = eng.minimize(bc)  # first launch (warm-up, counted in the complexities)
    t = time.perf_counter()
    flips = 0
    for _ in range(args.post_launches):
        bc = eng.minimize(bc)
        flips += int(eng.counters()["flips"].sum())
    t_min = time.perf_counter() - t
    rec = eng.records()
    ok = eng.validate(best=True)
    eng.close()
    log(f"minimizer {t_min:.2f} s, {flips} flips")
    runs, t_red, best_adds, naive_adds = 0, 0.0, [], []
    for m in np.unique(ranks):
        sel = np.nonzero(ranks == m)[0]
        coef = np.zeros((len(sel), 3, m, 64), np.int8)
        for c in range(3):
            bits = (rec.best_fac[sel][:, c, :m, None] >> np.arange(64, dtype=np.uint64)[None, None, :]) & np.uint64(1)
            coef[:, c, :, :nn[c]] = bits[:, :, :nn[c]].astype(np.int8)
        R = args.post_reducers
        red = fg.Reducer(n, int(m), coef, count=len(sel) * R, schemes=len(sel), seed=args.seed)
        tt = time.perf_counter()
        out = red.run()
        t_red += time.perf_counter() - tt
        red.close()
        runs += len(sel) * R
        adds = out["additions"].sum(axis=1).reshape(R, len(sel))  # reducer r reduces scheme r % schemes
        best_adds.append(adds.min(axis=0))
        naive_adds.append(out["naive"].sum(axis=1)[:len(sel)])
        log(f"rank {m}: {len(sel)} schemes, reducer total {t_red:.2f} s")
    best_adds, naive_adds = np.concatenate(best_adds), np.concatenate(naive_adds)
    print(json.dumps({
        "workload": f"post-search: complexity minimizer + additions reducer on {S} Z2 schemes of 4x4x4",
        "search_seconds": t_search, "ranks": {int(k): int(v) for k, v in zip(*np.unique(ranks, return_counts=True))},
        "schemes_valid": int(ok.sum()), "schemes_distinct": len({rec.best_fac[w].tobytes() for w in range(S)}),
        "minimizer": {"flips_per_s": flips / t_min if t_min > 0 else None, "flips": flips, "seconds": t_min,
                      "iterations": args.post_iterations, "launches": args.post_launches,
                      "complexity_start_mean": float(c0.mean()), "complexity_best_mean": float(bc.mean()),
                      "complexity_best_min": int(bc.min())},
        "reducer": {"runs": runs, "runs_per_s": runs / t_red, "seconds": t_red, "reducers_per_scheme": args.post_reducers,
                    "naive_additions_mean": float(naive_adds.mean()), "best_additions_mean": float(best_adds.mean()),
                    "best_additions_min": int(best_adds.min())}}))
    return 0


def zt_arm(args):
    """Integer-coefficient search: 16,384 walks per shape of (3,3,3) and (4,4,4) from the naive
    schemes, exact integer verification; verified flips/s and ranks reached.  Ternary (ZT, the
    reference's default ring) and Z2 in this engine's bit-exact reference mode, each beside the
    reference's own CUDA build on the same walks, steps and seed (ref_harness time, accepted flips
    counted by its twin kernel); then bounded by |c| <= 2 (ZB, fast mode)."""
    import flipgraphgpu_gb300 as fg
    for ring in ("zt", "z2"):
        for shape in ((3, 3, 3), (4, 4, 4)):
            n1, n2, n3 = shape
            eng = fg.Engine(args.zt_walks, n1 * n2 * n3, ring, "reference", args.seed, args.zt_iterations, 100000,
                            0.01, 0.0, 0, 0)
            eng.init_naive(n1, n2, n3)
            eng.run(1)
            tot_v, tot_ms = 0, 0.0
            for _ in range(args.steps):
                st = eng.run(1)
                tot_v += st["verified_flips"]
                tot_ms += st["kernel_ms"] + st["verify_ms"]
            c = eng.counters()
            eng.close()
            ours = tot_v / (tot_ms / 1000)
            ref = run_ref_harness(ring, ["time", args.zt_walks, args.zt_iterations, args.steps, args.seed, 100000,
                                         f"{n1}x{n2}x{n3}"], timeout=900)
            line = {"workload": f"{ring.upper()} {n1}x{n2}x{n3}, {args.zt_walks} walks, bit-exact reference mode",
                    "verified_flips_per_s": ours, "steps": args.steps, "iterations_per_step": args.zt_iterations,
                    "best_rank": int(c["best_rank"].min()), "walks_valid": int(c["valid"].sum())}
            if "unavailable" in ref:
                line["ref_cuda"] = ref
            else:
                line["ref_cuda"] = {"verified_flips_per_s": ref["verified_flips_per_s"],
                                    "ms_per_launch": ref["ms_per_launch"], "twin_mismatches": ref["twin_mismatches"],
                                    "valid_walks": ref["valid_walks"], "best_ranks": ref["best_ranks"]}
                line["ours_over_reference_cuda"] = ours / ref["verified_flips_per_s"]
            print(json.dumps(line))
            sys.stdout.flush()
    # Integer coefficients bounded by |c| <= 2 (fast mode; flips leaving the bound are rejected).
    for shape in ((3, 3, 3), (4, 4, 4)):
        n1, n2, n3 = shape
        full = n1 * n2 * n3
        eng = fg.Engine(args.zt_walks, full + 4, "zb", "fast", args.seed, args.zb_iterations, args.zb_plus, 0.01, 0.0)
        eng.init_naive(n1, n2, n3)
        eng.run(1)
        tot_v, tot_f, tot_ms = 0, 0, 0.0
        for _ in range(args.steps):
            st = eng.run(1)
            tot_v += st["verified_flips"]
            tot_f += st["flips"]
            tot_ms += st["kernel_ms"] + st["verify_ms"]
        c = eng.counters()
        proposals = args.steps * args.zb_iterations * args.zt_walks
        print(json.dumps({"workload": f"ZB (|c| <= 2) {n1}x{n2}x{n3}, {args.zt_walks} walks",
                          "verified_flips_per_s": tot_v / (tot_ms / 1000), "accepted_fraction": tot_f / proposals,
                          "steps": args.steps, "iterations_per_step": args.zb_iterations,
                          "plus_iterations": args.zb_plus, "best_rank": int(c["best_rank"].min()),
                          "walks_valid": int(c["valid"].sum())}))
        eng.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--walks", type=int, default=65536)
    ap.add_argument("--iterations", type=int, default=10000)
    ap.add_argument("--plus-iterations", type=int, default=100000)
    ap.add_argument("--mode", default="fast", choices=["fast", "philox", "reference"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--walks-per-block", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-iterations", type=int, default=100000, help="reference arm: steps per walk per step")
    ap.add_argument("--ref-walks-per-shape", type=int, default=64, help="reference arm: walks of each shape")
    ap.add_argument("--ref-cuda-launches", type=int, default=2, help="timed launches of the reference CUDA build")
    ap.add_argument("--no-extras", action="store_true", help="headline only: no ref_cuda, bitexact, ttr keys")
    ap.add_argument("--ttr-seeds", type=lambda x: [int(v) for v in x.split(",")], default=[1, 2, 3])
    ap.add_argument("--ttr444-seconds", type=float, default=60.0)
    ap.add_argument("--ttr-learned-records", type=int, default=2_000_000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--autotune", type=int, default=0, metavar="STEPS",
                    help="run fg_autotune with trials of STEPS steps before timing (0: the static kernel "
                         "choice, measured as fast as any tuned one on this workload)")
    ap.add_argument("--fast-kernel", default=None, choices=["auto", "thread", "group", "warp"],
                    help="fast mode: one kernel for every shape instead of the automatic choice")
    ap.add_argument("--lanes", type=int, default=0, help="group kernel: lanes per walk (4, 8, 16; 0 = by slots)")
    ap.add_argument("--fast-split", type=int, default=None,
                    help="fast mode: one thread per walk up to this many slots, one warp per walk above")
    ap.add_argument("--workload", default="batched", choices=["batched", "ttr", "zt", "learned", "post"])
    ap.add_argument("--post-schemes", type=int, default=4096)
    ap.add_argument("--post-iterations", type=int, default=2000)
    ap.add_argument("--post-launches", type=int, default=3)
    ap.add_argument("--post-reducers", type=int, default=32)
    ap.add_argument("--post-search-seconds", type=float, default=60.0)
    ap.add_argument("--learned-records", type=int, default=10_000_000)
    ap.add_argument("--learned-epochs", type=int, default=1)
    ap.add_argument("--learned-walks", type=int, default=65536)
    ap.add_argument("--learned-seconds", type=float, default=30.0)
    ap.add_argument("--learned-candidates", type=int, default=8)
    ap.add_argument("--learned-horizon", type=int, default=1000, help="label: rank drop within this many flips")
    ap.add_argument("--learned-every", type=int, default=16, help="record every n-th accepted flip")
    ap.add_argument("--ttr-modes", default="fast,reference")
    ap.add_argument("--ttr-seconds", type=float, default=300.0)
    ap.add_argument("--ttr-shape", default="3x3x3")
    ap.add_argument("--ttr-target", type=int, default=23)
    ap.add_argument("--ttr-walks", type=int, default=1024)
    ap.add_argument("--ttr-iterations", type=int, default=1000)
    ap.add_argument("--ttr-plus", type=int, default=50000)
    ap.add_argument("--zt-walks", type=int, default=16384)
    ap.add_argument("--zt-iterations", type=int, default=200)
    ap.add_argument("--zb-iterations", type=int, default=2000)
    ap.add_argument("--zb-plus", type=int, default=5000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "ttr":
        return ttr_arm(args)
    if args.workload == "zt":
        return zt_arm(args)
    if args.workload == "learned":
        return learned_arm(args)
    if args.workload == "post":
        return post_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
