"""Benchmark: exact sorted-u32 pair intersection on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one step): the skewed 2-set sweep -- four independent pairs with
|large| = 2^24 and |small| in {2^10, 2^14, 2^18, 2^24}, element space
m = |large| / 0.05, selectivity 1% of |small|, seeded synthetic data shaped
like the reference's generator (benchmark/src/generators.rs:30-68).  Each
pair is intersected exactly (materialised, ascending) with the algorithm the
policy picks for its size ratio.

* ``value``: pair intersections/s with inputs resident in HBM (device
  pointers, async C-ABI calls; the K steps captured once into a CUDA graph,
  the steady-state form), timed with CUDA events over one replay.
* ``e2e``: the same through the host-pointer C-ABI call
  (``setops_gpu_intersect(..., SETOPS_HOST)``): pinned host inputs copied in
  and the result copied out inside the timed region.
* ``roofline``: the kernel the policy picks for the 2^24 x 2^24 pair (the
  tiled bitmap kernel); algorithmic
  bytes = both inputs read + output written, over its CUDA-event time.
* ``cpu_baseline``: the reference's CPU path (oracle port: best of
  shuffling / SIMD galloping / bmiss per pair) on this host's cores.

* ``serve``: the serving configuration -- k-set queries against a resident
  index of 1M posting lists, Poisson arrivals at several rates, queries/s
  with p50/p99 latency, beside one k-set call per query.
* ``batch``: the batched configuration -- 100,000 uneven pairs in one
  persistent launch (policy autotuned on a sample) against one launch per
  pair on a sample of the same pairs; results checked equal.

``--impl reference`` times that CPU path alone on all host threads (pairs
spread over threads), rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pair intersections/sec & GB/s vs HBM peak (exact)"
UNIT = "pair-intersections/s"
SMALL_EXPS = (10, 14, 18, 24)
LARGE = 1 << 24
DENSITY = 0.05
SELECTIVITY = 0.01
SEED = 20240601


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--cpu-sample-seconds", type=float, default=10.0)
    p.add_argument("--min-warmup-seconds", type=float, default=2.0,
                   help="keep warming up at least this long (gives the clock sampler "
                        "load to observe)")
    p.add_argument("--no-batch", action="store_true",
                   help="skip the batched-pairs leg (100k uneven pairs in one launch)")
    p.add_argument("--batch-pairs", type=int, default=100000)
    p.add_argument("--bsr-pairs", type=int, default=10000,
                   help="pairs of the BSR subset of the batch leg")
    p.add_argument("--no-kset", action="store_true", help="skip the k-set leg")
    p.add_argument("--kset-ks", default="3,5,8", help="k values of the k-set leg")
    p.add_argument("--no-graph", action="store_true",
                   help="time the sweep's calls directly instead of one CUDA-graph replay")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the hand-written policy table (no tuning before the sweep)")
    p.add_argument("--no-config0", action="store_true",
                   help="skip the plain 2^20 x 2^20 pair leg")
    p.add_argument("--no-serve", action="store_true",
                   help="skip the serving leg (k-set queries against a resident index)")
    p.add_argument("--serve-rates", default="10000,50000,200000,1000000",
                   help="Poisson arrival rates (queries/s) of the serving leg")
    p.add_argument("--pairs", default="0,1,2,3",
                   help="which sweep pairs to run (profiling subsets; default all)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def sweep_seeds(rank: int) -> list[int]:
    """Seeds of a rank's sweep pairs: every rank (replica) intersects its own
    pairs of the same shapes; rank 0's are the single-GPU workload."""
    return [SEED + 1000 * rank + k for k in range(len(SMALL_EXPS))]


def make_sweep(rank: int, ds=None):
    if ds is None:
        from simd_set_operations_gb300 import datasets as ds
    return [ds.gen_twoset(sd, DENSITY, SELECTIVITY, 1 << e, LARGE)
            for sd, e in zip(sweep_seeds(rank), SMALL_EXPS)]


def cpu_datasets():
    """The input generators for a CPU-only process: datasets.py loaded on its
    own (not through the package, whose import maps the GPU library) and
    bound to the oracle's library, which is built from the same generator
    source and so makes the same inputs."""
    import importlib.util

    import oracle
    name = "setops_cpu_datasets"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, ROOT / "simd_set_operations_gb300" / "datasets.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    mod.use_library(oracle.lib())
    return mod


def max_over_ranks(x: float) -> float:
    """The largest x over the ranks (a timed region's length: the job ends
    with its slowest rank); x itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, pairs_per_step: int, steps: int, seconds: float) -> float:
    """Whole-job throughput: the pairs every rank intersected over the
    slowest rank's time (weak scaling: per-rank work fixed)."""
    return world * pairs_per_step * steps / seconds


def algorithmic_bytes(ns: int, nl: int, nout: int) -> int:
    return 4 * (ns + nl) + 4 * nout


def touched_bytes(ns: int, nl: int, nout: int) -> int:
    """Estimated bytes a search-band pair really moves: the small set read,
    the output written, and in the large set the 32-byte sectors its probes
    touch.  A search for one small element narrows a gap of about nl/ns
    elements; the levels whose probes are more than one sector (8 elements)
    apart each touch a sector of their own, the last ones share one:
    max(1, ceil(log2(nl/ns)) - 2) sectors per element, capped at the whole
    large set."""
    import math
    per = max(1, math.ceil(math.log2(max(nl / max(ns, 1), 2))) - 2)
    return 4 * ns + 4 * nout + min(32 * per * ns, 4 * nl)


def workload_config(sel=None):
    cfg = {
        "workload": "skewed 2-set sweep: |large| = 2^24, |small| in {2^10, 2^14, 2^18, 2^24}, "
                    "density 0.05, selectivity 0.01, materialised sorted output",
        "pairs_per_step": len(SMALL_EXPS),
        "small_sizes": [1 << e for e in SMALL_EXPS],
        "large_size": LARGE,
        "element_space": int(LARGE / DENSITY),
        "density": DENSITY,
        "selectivity": SELECTIVITY,
        "seed": SEED,
        "l2": "inputs larger than L2: 321 MiB read per step vs 129 MB L2, each array "
              "touched once per step; no flush",
    }
    if sel is not None and len(sel) != len(SMALL_EXPS):
        cfg["pairs_run"] = [1 << SMALL_EXPS[i] for i in sel]
    return cfg


# ---------------------------------------------------------------------------
# clocks

CLOCK_Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"setops_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={CLOCK_Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        try:
            self.path.unlink()
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power) if power else None, "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU path (oracle port of the reference's CPU algorithms)

def cpu_sweep_best(pairs, nthreads: int, seconds: float):
    """Times each baseline on each pair (pairs spread over `nthreads`
    threads), picks the best algorithm per pair, and returns (pairs/s for a
    full sweep with the best per-pair algorithms, details)."""
    import oracle
    algos = [oracle.SHUFFLING_W8, oracle.SIMD_GALLOPING_W16, oracle.BMISS_W4]
    outs = [np.empty(min(s.size, l.size), np.uint32) for s, l in pairs]
    best = []
    t_total = 0.0
    counts = None
    for i, (s, l) in enumerate(pairs):
        times = {}
        for a in algos:
            reps, t0 = 0, time.perf_counter()
            while True:
                c = oracle.run_pairs(a, [(s, l)], 1, outs=[outs[i]])
                reps += 1
                el = time.perf_counter() - t0
                if el > seconds / (len(pairs) * len(algos)) or reps >= 50:
                    break
            times[a] = el / reps
            t_total += el
        a = min(times, key=times.get)
        best.append((a, times[a], times))
    # full sweep with best algorithm per pair, pairs spread over threads
    groups = {}
    for i, (a, _, _) in enumerate(best):
        groups.setdefault(a, []).append(i)
    reps, t0 = 0, time.perf_counter()
    while True:
        if nthreads > 1:
            import threading
            res = {}

            def run(a, idx):
                res[a] = oracle.run_pairs(a, [pairs[i] for i in idx], len(idx))
            ths = [threading.Thread(target=run, args=(a, idx)) for a, idx in groups.items()]
            for t in ths:
                t.start()
            for t in ths:
                t.join()
        else:
            res = {a: oracle.run_pairs(a, [pairs[i] for i in idx], 1) for a, idx in groups.items()}
        reps += 1
        el = time.perf_counter() - t0
        if el > max(1.0, seconds / 4) or reps >= 20:
            break
    counts = [0] * len(pairs)
    for a, idx in groups.items():
        for j, i in enumerate(idx):
            counts[i] = int(res[a][j])
    sweep_s = el / reps
    detail = [{"small": int(s.size), "large": int(l.size),
               "best": oracle.ALGO_NAMES[a], "seconds": t,
               "all": {oracle.ALGO_NAMES[k]: v for k, v in tt.items()}}
              for (s, l), (a, t, tt) in zip(pairs, best)]
    return len(pairs) / sweep_s, sweep_s, detail, counts, outs, t_total + el


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.lib()
    cores = oracle.host_cores()
    pairs = make_sweep(0, cpu_datasets())
    # warmup: algorithm choice per pair (bounded)
    _, _, detail, _, _, _ = cpu_sweep_best(pairs, 1, min(args.cpu_sample_seconds, 6.0))
    best = [next(k for k, v in oracle.ALGO_NAMES.items() if v == d["best"]) for d in detail]
    groups = {}
    for i, a in enumerate(best):
        groups.setdefault(a, []).append(i)
    import threading

    def sweep():
        res = {}

        def run(a, idx):
            res[a] = oracle.run_pairs(a, [pairs[i] for i in idx], max(1, min(len(idx), cores)))
        ths = [threading.Thread(target=run, args=(a, idx)) for a, idx in groups.items()]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        return res

    for _ in range(max(args.warmup, 1)):
        sweep()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sweep()
    el = time.perf_counter() - t0
    value = len(pairs) * args.steps / el
    used = min(cores, len(pairs))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic", "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": used, "kind": "port",
                         "sample": f"{args.steps} full sweeps (4 pairs each), best algorithm per "
                                   "pair, pairs spread over threads",
                         "algorithms": detail, "host_cores": cores,
                         "arch": os.uname().machine},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm

def read_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def read_traffic():
    """DRAM bytes per launch of the headline kernel from the committed ncu
    summary (profiles/), or None."""
    f = ROOT / "profiles" / "awindow_2e24x2e24_ncu.md"
    if not f.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9]+)", f.read_text())
    return int(m.group(1)) if m else None


CONFIG0_SEED = 20240620


def cpu_best_single_pair(a, b, seconds: float) -> dict:
    """The reference's CPU path on one pair: each baseline (shuffling, SIMD
    galloping, bmiss) timed single-core for about seconds/3, best kept; and
    all cores, which the reference can only use on separate pairs, timed on
    one copy of the pair per thread."""
    import oracle
    cores = oracle.host_cores()
    out = np.empty(min(a.size, b.size), np.uint32)
    per = {}
    for algo in (oracle.SHUFFLING_W8, oracle.SIMD_GALLOPING_W16, oracle.BMISS_W4):
        reps, t0 = 0, time.perf_counter()
        while True:
            oracle.run_pairs(algo, [(a, b)], 1, outs=[out])
            reps += 1
            el = time.perf_counter() - t0
            if el > seconds / 3 or reps >= 200:
                break
        per[oracle.ALGO_NAMES[algo]] = el / reps
    best_name = min(per, key=per.get)
    best = next(k for k, v in oracle.ALGO_NAMES.items() if v == best_name)
    reps, t0 = 0, time.perf_counter()
    while True:
        oracle.run_pairs(best, [(a, b)] * cores, cores)
        reps += 1
        el = time.perf_counter() - t0
        if el > max(0.5, seconds / 4) or reps >= 50:
            break
    return {"single_core": {"value": 1.0 / per[best_name], "cores": 1, "seconds_per_pair":
                            per[best_name], "best": best_name, "all": per},
            "all_cores": {"value": cores * reps / el, "cores": cores,
                          "sample": f"{cores} copies of the pair, one per thread, {reps} rounds"},
            "arch": os.uname().machine}


def config0_leg(ctx, stream, cpu_seconds: float, with_cpu: bool) -> dict:
    """The plain 2-set configuration: |A| = |B| = 2^20, element space
    2^20 / 0.1, selectivity 0.1 (the reference's gen_twoset shape,
    benchmark/src/generators.rs:30-68).  Materialised and counted on resident
    inputs (CUDA events over 50 back-to-back launches), end to end through
    the host-pointer call with copies, and the CPU path beside it; the GPU
    result must equal naive_merge."""
    import ctypes as C

    import torch

    import oracle
    from simd_set_operations_gb300 import _lib, datasets as ds
    L = _lib.lib
    n = 1 << 20
    a, b = ds.gen_twoset(CONFIG0_SEED, 0.1, 0.1, n, n)
    want = oracle.naive_merge(a, b)
    # 24 copies of the pair (192 MiB, more than the 129 MB L2), launches
    # rotating over them so that each launch reads its inputs from HBM
    ncopy = 24
    da = torch.from_numpy(a.view(np.int32)).cuda()
    db = torch.from_numpy(b.view(np.int32)).cuda()
    copies = [(da, db)] + [(da.clone(), db.clone()) for _ in range(ncopy - 1)]
    outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(ncopy)]
    ln = torch.zeros(2 * ncopy, dtype=torch.int64, device="cuda")
    h = ctx.handle

    def launch(i: int, mat: bool):
        x, y = copies[i % ncopy]
        rc = L.setops_gpu_intersect_async(h, x.data_ptr(), n, y.data_ptr(), n,
                                          outs[i % ncopy].data_ptr() if mat else None, n,
                                          ln.data_ptr() + 8 * (2 * (i % ncopy) + (0 if mat else 1)),
                                          0)
        if rc != 0:
            ctx.check(rc)

    res = {}
    for mat in (True, False):
        for i in range(ncopy):
            launch(i, mat)
        ts = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(2 * ncopy):
                launch(i, mat)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / (2 * ncopy))
        res["materialise" if mat else "count"] = min(ts), statistics.mean(ts)
    ctx.synchronize()
    lens_all = ln.cpu().numpy()
    if not np.all(lens_all == want.size):
        raise SystemExit("config 0: a copy's GPU result length differs from naive_merge")
    got = outs[ncopy - 1][:want.size].cpu().numpy().view(np.uint32)
    del copies, outs
    if not np.array_equal(got, want):
        raise SystemExit("config 0: GPU result differs from naive_merge")
    # end to end: pinned host buffers through setops_gpu_intersect(..., HOST)
    pa = torch.from_numpy(a.view(np.int32)).pin_memory().numpy().view(np.uint32)
    pb = torch.from_numpy(b.view(np.int32)).pin_memory().numpy().view(np.uint32)
    po = torch.empty(n, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    nout = C.c_size_t()

    def e2e_call():
        ctx.check(L.setops_gpu_intersect(h, pa.ctypes.data, n, pb.ctypes.data, n, po.ctypes.data,
                                         n, C.byref(nout), _lib.HOST))
    for _ in range(3):
        e2e_call()
    reps = 30
    t0 = time.perf_counter()
    for _ in range(reps):
        e2e_call()
    e_el = (time.perf_counter() - t0) / reps
    if nout.value != want.size or not np.array_equal(po[:want.size], want):
        raise SystemExit("config 0: host-pointer result differs from naive_merge")
    peak, kind = read_peak()
    alg = 4 * 2 * n + 4 * want.size
    ms = res["materialise"][1]
    line = {
        "workload": "plain 2-set pair: |A| = |B| = 2^20, element space 2^20 / 0.1, selectivity "
                    "0.1, u32, materialised sorted output; checked equal to naive_merge",
        "seed": CONFIG0_SEED, "out": int(want.size),
        "pairs_per_s": 1e3 / ms, "ms": ms, "ms_min": res["materialise"][0],
        "count_ms": res["count"][1],
        "algorithmic_bytes": alg, "GBps_algorithmic": alg / (ms / 1e3) / 1e9,
        "frac_of_peak": alg / (ms / 1e3) / 1e9 / peak, "peak_source": f"{kind} (hbm_gbs)",
        "l2": "launches rotate over 24 device copies of the pair (192 MiB > 129 MB L2)",
        "e2e": {"pairs_per_s": 1.0 / e_el, "ms_per_pair": 1e3 * e_el,
                "h2d_bytes_per_pair": 8 * n, "d2h_bytes_per_pair": 4 * int(want.size) + 8,
                "api": "setops_gpu_intersect(..., SETOPS_HOST), pinned host buffers"},
        "results_match_naive_merge": True,
    }
    if with_cpu:
        cpu = cpu_best_single_pair(a, b, cpu_seconds)
        line["cpu_baseline"] = {"value": cpu["single_core"]["value"], "unit": "pairs/s",
                                "cores": 1, "kind": "port", **cpu}
    return line


BATCH_SEED = 20240611


def cpu_pairs_baseline(pairs, cores: int, caps) -> dict:
    """The reference's CPU path over a batch of pairs: each baseline
    (shuffling, SIMD galloping, bmiss) over every pair on all cores (pairs
    spread over threads), best kept; and single-core on a 2,000-pair sample,
    scaled to pairs/s."""
    import oracle
    outs = [np.empty(max(int(c), 1), np.uint32) for c in caps]
    algos = (oracle.SHUFFLING_W8, oracle.SIMD_GALLOPING_W16, oracle.BMISS_W4)
    allc, single = {}, {}
    ns = min(len(pairs), 2000)
    for algo in algos:
        oracle.run_pairs(algo, pairs[:ns], cores, outs=outs[:ns])  # warm-up
        t0 = time.perf_counter()
        oracle.run_pairs(algo, pairs, cores, outs=outs)
        allc[oracle.ALGO_NAMES[algo]] = len(pairs) / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.run_pairs(algo, pairs[:ns], 1, outs=outs[:ns])
        single[oracle.ALGO_NAMES[algo]] = ns / (time.perf_counter() - t0)
    best = max(allc, key=allc.get)
    return {"value": allc[best], "unit": "pairs/s", "cores": cores, "kind": "port",
            "best": best, "all_cores": allc,
            "single_core": {"value": max(single.values()), "cores": 1,
                            "best": max(single, key=single.get), "all": single,
                            "sample_pairs": ns},
            "sample": f"all {len(pairs)} pairs per baseline on {cores} threads",
            "arch": os.uname().machine}


def batch_leg(ctx, stream, npairs: int) -> dict:
    """Batched uneven pairs (the reference's batched configuration): npairs
    pairs with set sizes log-uniform in [2^4, 2^16], per-pair density
    U[0.01, 0.5] and selectivity U[0, 0.5], intersected in one launch from
    device-resident data, against the plain path of one launch per pair on a
    sample of the same pairs.  The batch policy is first autotuned on the
    first 10,000 pairs.  The per-pair results of the sample must equal the
    batch's."""
    import ctypes as C

    import torch

    from simd_set_operations_gb300 import _lib, datasets as ds
    L = _lib.lib
    b = ds.gen_batch(BATCH_SEED, npairs, 16, 1 << 16)
    td = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()  # noqa: E731
    pool = td(b.pool, np.int32)
    arrs = [td(x, np.int64) for x in (b.a_off, b.a_len, b.b_off, b.b_len)]
    caps = np.minimum(b.a_len, b.b_len)
    cap = int(caps.sum())
    offs = np.zeros(npairs, np.uint64)
    offs[1:] = np.cumsum(caps[:-1])
    doffs = td(offs, np.int64)
    out = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    lens = torch.zeros(npairs, dtype=torch.int64, device="cuda")
    # autotune the batch policy on the batch itself (device arrays; a 10,000-
    # pair sample once chose a search ratio that was 20 % slower on the whole)
    nt = npairs
    ctx.check(L.setops_gpu_batch_autotune(ctx.handle, pool.data_ptr(), pool.numel(),
                                          *[a.data_ptr() for a in arrs], nt, 3, 0))
    v, r = C.c_int(), C.c_uint32()
    ctx.check(L.setops_gpu_batch_get_policy(ctx.handle, C.byref(v), C.byref(r)))

    def run():
        ctx.check(L.setops_gpu_batch_intersect(
            ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], npairs,
            out.data_ptr(), cap, doffs.data_ptr(), lens.data_ptr(), 0))

    for _ in range(2):
        run()
    ts = []
    for _ in range(7):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t_batch = sorted(ts)[len(ts) // 2]
    matches = int(lens.sum().item())
    alg = 4 * int(b.pool.size) + 4 * matches
    steady = steady_state(ctx, stream, L, pool, arrs, npairs, out, cap, doffs, lens)
    # the plain path: one launch per pair (async C-ABI on device pointers),
    # looped in C over every pair of the batch
    out2 = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    ln2 = torch.zeros(npairs, dtype=torch.int64, device="cuda")
    secs = C.c_double()

    def per_pair():
        ctx.check(L.setops_bench_pairs_one_by_one(
            ctx.handle, pool.data_ptr(), b.a_off.ctypes.data, b.a_len.ctypes.data,
            b.b_off.ctypes.data, b.b_len.ctypes.data, npairs, out2.data_ptr(),
            offs.ctypes.data, ln2.data_ptr(), C.byref(secs)))
        return secs.value

    per_pair()
    t_pp = min(per_pair() for _ in range(2))
    # exactness: every pair of the batch equals the per-pair path and the
    # oracle's naive_merge
    import oracle
    cores = oracle.host_cores()
    l1, l2 = lens.cpu().numpy(), ln2.cpu().numpy()
    o1, o2 = out.cpu().numpy().view(np.uint32), out2.cpu().numpy().view(np.uint32)
    pairs = [b.pair(p) for p in range(npairs)]
    exp = np.zeros(max(cap, 1), np.uint32)
    views = [exp[int(offs[p]):int(offs[p]) + max(int(caps[p]), 0)] for p in range(npairs)]
    t0 = time.perf_counter()
    wl = oracle.run_pairs(oracle.NAIVE_MERGE, pairs, cores,
                          outs=[v if v.size else exp[:1] for v in views])
    t_oracle = time.perf_counter() - t0
    mask = np.zeros(max(cap, 1) + 1, np.int64)
    np.add.at(mask, offs.astype(np.int64), 1)
    np.add.at(mask, (offs + wl).astype(np.int64), -1)
    mask = np.cumsum(mask)[:max(cap, 1)] > 0
    if not (np.array_equal(l1, wl.astype(np.int64)) and np.array_equal(l2, l1)):
        raise SystemExit("batch: result lengths differ from naive_merge or the per-pair path")
    if not (np.array_equal(o1[mask], exp[mask]) and np.array_equal(o2[mask], exp[mask])):
        raise SystemExit("batch: results differ from naive_merge or the per-pair path")
    cpu = cpu_pairs_baseline(pairs, cores, caps)
    peak, _ = read_peak()
    return {
        "workload": f"{npairs} pairs, sizes log-uniform in [2^4, 2^16] per set, density "
                    "U[0.01, 0.5], selectivity U[0, 0.5], u32, materialised; inputs resident",
        "pairs": npairs, "pool_bytes": 4 * int(b.pool.size), "matches": matches,
        "ms": 1e3 * t_batch, "pairs_per_s": npairs / t_batch,
        "GBps_algorithmic": alg / t_batch / 1e9, "frac_of_peak": alg / t_batch / 1e9 / peak,
        "policy": {"variant": int(v.value), "search_ratio": int(r.value),
                   "tuned_on_pairs": nt},
        "one_launch_per_pair": {"pairs_per_s": npairs / t_pp, "pairs": npairs,
                                "api": "setops_gpu_intersect_async per pair on device pointers, "
                                       "looped in C (setops_bench_pairs_one_by_one)"},
        "speedup_vs_one_launch_per_pair": (npairs / t_batch) / (npairs / t_pp),
        "results_match_per_pair_path": True,
        "results_match_naive_merge": f"all {npairs} pairs (oracle, {cores} threads, "
                                     f"{t_oracle:.1f} s)",
        "cpu_baseline": cpu,
        "steady_state": steady,
    }


def steady_state(ctx, stream, L, pool, arrs, npairs, out, cap, doffs, lens) -> dict:
    """Steady-state launches: a batch plan (the batch captured once in a CUDA
    graph) replayed back to back, against repeated plain batch calls on the
    same device arrays (each call: offset scan, capacity read-back, launch).
    For the whole batch and for its first 1,000 pairs.  Replays must give the
    plain call's results."""
    import ctypes as C

    import torch

    res = {"api": "setops_gpu_batch_plan_create / _launch vs setops_gpu_batch_intersect"}
    for label, n in (("full", npairs), ("small", min(1000, npairs))):
        reps = 5 if label == "full" else 50
        sub_cap = cap if n == npairs else int(doffs[n].item())
        plan = C.c_void_p()
        ctx.check(L.setops_gpu_batch_plan_create(
            ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
            out.data_ptr(), sub_cap, None, lens.data_ptr(), C.byref(plan)))
        try:
            ctx.check(L.setops_gpu_batch_plan_launch(plan))
            ctx.check(L.setops_gpu_synchronize(ctx.handle))
            ref_out = out[:sub_cap].clone()
            ref_lens = lens[:n].clone()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                ctx.check(L.setops_gpu_batch_plan_launch(plan))
            e1.record(stream)
            e1.synchronize()
            ctx.check(L.setops_gpu_synchronize(ctx.handle))
            t_graph = e0.elapsed_time(e1) * 1e-3 / reps
        finally:
            ctx.check(L.setops_gpu_batch_plan_destroy(plan))

        def plain():
            ctx.check(L.setops_gpu_batch_intersect(
                ctx.handle, pool.data_ptr(), pool.numel(), *[a.data_ptr() for a in arrs], n,
                out.data_ptr(), sub_cap, None, lens.data_ptr(), 0))
        plain()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            plain()
        torch.cuda.synchronize()
        t_plain = (time.perf_counter() - t0) / reps
        if not (torch.equal(ref_lens, lens[:n]) and torch.equal(ref_out, out[:sub_cap])):
            raise SystemExit(f"graph replay of the {label} batch differs from the plain call")
        res[label] = {"pairs": n, "replays": reps, "graph_ms": 1e3 * t_graph,
                      "plain_call_ms": 1e3 * t_plain, "graph_pairs_per_s": n / t_graph,
                      "speedup": t_plain / t_graph, "results_equal": True}
    return res


BSR_SEED = 20240617


def batch_bsr_leg(ctx, stream, npairs: int) -> dict:
    """The batched configuration's BSR subset: npairs pairs at density 0.5
    (sizes log-uniform in [2^4, 2^16] elements, selectivity U[0, 0.5]),
    encoded as BSR words (32-bit base + 32-bit state; encoding outside the
    timed region, as in the reference's harness) and intersected in one
    launch, against one setops_gpu_intersect_bsr call per pair on a sample;
    the sample's per-pair results must equal the batch's."""
    import ctypes as C

    import torch

    from simd_set_operations_gb300 import _lib, datasets as ds
    L = _lib.lib
    bb = ds.bsr_encode_batch(ds.gen_batch(BSR_SEED, npairs, 16, 1 << 16, density=(0.5, 0.5)))
    td = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x).view(dt)).cuda()  # noqa: E731
    bases, states = td(bb.bases, np.int32), td(bb.states, np.int32)
    arrs = [td(x, np.int64) for x in (bb.a_off, bb.a_len, bb.b_off, bb.b_len)]
    caps = np.minimum(bb.a_len, bb.b_len)
    cap = max(int(caps.sum()), 1)
    offs = np.zeros(npairs, np.uint64)
    offs[1:] = np.cumsum(caps[:-1])
    doffs = td(offs, np.int64)
    ob = torch.empty(cap, dtype=torch.int32, device="cuda")
    os_ = torch.empty(cap, dtype=torch.int32, device="cuda")
    lens = torch.zeros(npairs, dtype=torch.int64, device="cuda")

    def run():
        ctx.check(L.setops_gpu_batch_intersect_bsr(
            ctx.handle, bases.data_ptr(), states.data_ptr(), bases.numel(),
            *[a.data_ptr() for a in arrs], npairs, ob.data_ptr(), os_.data_ptr(), cap,
            doffs.data_ptr(), lens.data_ptr(), 0))

    for _ in range(2):
        run()
    ts = []
    for _ in range(7):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t_batch = sorted(ts)[len(ts) // 2]
    words_out = int(lens.sum().item())
    alg = 8 * (int(bb.a_len.sum()) + int(bb.b_len.sum())) + 8 * words_out
    # the plain path: one BSR call per pair (device pointers), looped in C
    # over every pair
    hb, hs, hl = ob.cpu().numpy().view(np.uint32), os_.cpu().numpy().view(np.uint32), lens.cpu().numpy()
    ob2 = torch.empty(cap, dtype=torch.int32, device="cuda")
    os2 = torch.empty_like(ob2)
    hl2 = np.zeros(npairs, np.uint64)
    secs = C.c_double()

    def per_pair():
        ctx.check(L.setops_bench_bsr_pairs_one_by_one(
            ctx.handle, bases.data_ptr(), states.data_ptr(), bb.a_off.ctypes.data,
            bb.a_len.ctypes.data, bb.b_off.ctypes.data, bb.b_len.ctypes.data, npairs,
            ob2.data_ptr(), os2.data_ptr(), offs.ctypes.data, hl2.ctypes.data, C.byref(secs)))
        return secs.value

    per_pair()
    t_pp = min(per_pair() for _ in range(2))
    # exactness: every pair equals the per-pair path and the oracle's
    # branchless_merge_bsr
    import oracle
    cores = oracle.host_cores()
    pairs = [bb.pair(p) for p in range(npairs)]
    eb, es = np.zeros(cap, np.uint32), np.zeros(cap, np.uint32)
    vo = [(eb[int(offs[p]):int(offs[p]) + max(int(caps[p]), 1)],
           es[int(offs[p]):int(offs[p]) + max(int(caps[p]), 1)]) for p in range(npairs)]
    eb_pad = np.zeros(1, np.uint32)
    vo = [v if v[0].size else (eb_pad, eb_pad.copy()) for v in vo]
    wl = oracle.run_bsr_pairs(pairs, cores, outs=vo)
    mask = np.zeros(cap + 1, np.int64)
    np.add.at(mask, offs.astype(np.int64), 1)
    np.add.at(mask, (offs + wl).astype(np.int64), -1)
    mask = np.cumsum(mask)[:cap] > 0
    hb2, hs2 = ob2.cpu().numpy().view(np.uint32), os2.cpu().numpy().view(np.uint32)
    if not (np.array_equal(hl.astype(np.uint64), wl) and np.array_equal(hl2, wl)):
        raise SystemExit("BSR batch: result lengths differ from branchless_merge_bsr")
    if not all(np.array_equal(x[mask], y[mask]) for x, y in
               ((hb, eb), (hs, es), (hb2, eb), (hs2, es))):
        raise SystemExit("BSR batch: results differ from branchless_merge_bsr")
    allc, single = {}, {}
    ns = min(npairs, 2000)
    for algo, name in ((0, "branchless_merge_bsr"), (1, "galloping_bsr")):
        oracle.run_bsr_pairs(pairs[:ns], cores, algo=algo)
        t0 = time.perf_counter()
        oracle.run_bsr_pairs(pairs, cores, algo=algo)
        allc[name] = npairs / (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.run_bsr_pairs(pairs[:ns], 1, algo=algo)
        single[name] = ns / (time.perf_counter() - t0)
    best = max(allc, key=allc.get)
    cpu = {"value": allc[best], "unit": "pairs/s", "cores": cores, "kind": "port", "best": best,
           "all_cores": allc, "single_core": {"value": max(single.values()), "cores": 1,
                                              "all": single, "sample_pairs": ns},
           "sample": f"all {npairs} BSR pairs per baseline on {cores} threads (count only)",
           "arch": os.uname().machine}
    peak, _ = read_peak()
    return {
        "workload": f"{npairs} BSR pairs at density 0.5 (sizes log-uniform in [2^4, 2^16] "
                    "elements, selectivity U[0, 0.5]), 32-bit base + 32-bit state words, "
                    "materialised; inputs resident",
        "pairs": npairs, "words_in": int(bb.a_len.sum()) + int(bb.b_len.sum()),
        "words_out": words_out, "ms": 1e3 * t_batch, "pairs_per_s": npairs / t_batch,
        "GBps_algorithmic": alg / t_batch / 1e9, "frac_of_peak": alg / t_batch / 1e9 / peak,
        "one_call_per_pair": {"pairs_per_s": npairs / t_pp, "pairs": npairs,
                              "api": "setops_gpu_intersect_bsr per pair on device pointers, "
                                     "looped in C (setops_bench_bsr_pairs_one_by_one)"},
        "speedup_vs_one_call_per_pair": (npairs / t_batch) / (npairs / t_pp),
        "results_match_per_pair_path": True,
        "results_match_branchless_merge_bsr": f"all {npairs} pairs",
        "cpu_baseline": cpu,
    }


KSET_SEED = 20240618


def cpu_kset_baseline(sets, nout: int) -> dict:
    """The reference's CPU k-set path (svs_generic, smallest first) with each
    baseline as its 2-set function: single-core best (timed for about a
    second each), and all cores on one copy of the group per thread."""
    import oracle
    cores = oracle.host_cores()
    outs = [np.empty(max(min(x.size for x in sets), 1), np.uint32)]
    per = {}
    for algo in (oracle.SHUFFLING_W8, oracle.SIMD_GALLOPING_W16, oracle.BMISS_W4):
        reps, t0 = 0, time.perf_counter()
        while True:
            c = oracle.run_svs_groups([sets], 1, outs=outs, algo=algo)
            reps += 1
            el = time.perf_counter() - t0
            if el > 1.0 or reps >= 100:
                break
        if int(c[0]) != nout:
            raise SystemExit("CPU k-set baseline disagrees with svs_generic")
        per[oracle.ALGO_NAMES[algo]] = reps / el
    best_name = max(per, key=per.get)
    best = next(k for k, v in oracle.ALGO_NAMES.items() if v == best_name)
    reps, t0 = 0, time.perf_counter()
    while True:
        oracle.run_svs_groups([sets] * cores, cores, algo=best)
        reps += 1
        el = time.perf_counter() - t0
        if el > 1.0 or reps >= 50:
            break
    return {"value": cores * reps / el, "unit": "k-sets/s", "cores": cores, "kind": "port",
            "sample": f"{cores} copies of the k-set, one per thread, {reps} rounds",
            "best": best_name,
            "single_core": {"value": per[best_name], "cores": 1, "all": per},
            "arch": os.uname().machine}


def kset_leg(ctx, stream, ks=(3, 5, 8), with_cpu: bool = True) -> dict:
    """The reference's k-set configuration: k sorted sets with |S_1| = 2^22
    and Zipf sizes |S_i| = 2^22 / i (exponent 1.0, the reference's skewness
    factor 1000 in thousandths), element space
    2^22 / 0.2, a core of 5 % of the smallest set in every set, intersected
    smallest-first (svs_generic, setops/src/intersect/svs.rs:50-73) with the
    intermediates on the device: setops_gpu_svs on device pointers, CUDA
    events over back-to-back calls.  Algorithmic bytes: every set read once
    plus the output written."""
    import ctypes as C

    import torch

    from simd_set_operations_gb300 import _lib, datasets as ds
    L = _lib.lib
    peak, _ = read_peak()
    rows = []
    for k in ks:
        sets = ds.gen_kset(KSET_SEED + k, 0.2, 0.05, 1 << 22, 1.0, k)  # Zipf exponent 1.0
        dsets = [torch.from_numpy(x.view(np.int32)).cuda() for x in sets]
        ptrs = (C.c_void_p * k)(*[d.data_ptr() for d in dsets])
        lens = (C.c_size_t * k)(*[int(x.size) for x in sets])
        cap = min(int(x.size) for x in sets)
        out = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
        n_out = C.c_size_t()

        dlen = torch.zeros(1, dtype=torch.int64, device="cuda")

        def run():
            ctx.check(L.setops_gpu_svs(ctx.handle, ptrs, lens, k, out.data_ptr(), out.numel(),
                                       C.byref(n_out), 0))

        def run_async():  # back-to-back: the length stays on the device
            ctx.check(L.setops_gpu_svs_async(ctx.handle, ptrs, lens, k, out.data_ptr(),
                                             out.numel(), dlen.data_ptr(), 0))
        for _ in range(3):
            run()
            run_async()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(20):
            run_async()
        e1.record(stream)
        e1.synchronize()
        ctx.check(L.setops_gpu_synchronize(ctx.handle))
        t_dev = e0.elapsed_time(e1) * 1e-3 / 20
        if int(dlen.item()) != int(n_out.value):
            raise SystemExit(f"k={k}: the asynchronous call gave {int(dlen.item())} results")
        # the same call captured once in a CUDA graph and replayed: device time
        # without the host work of each call
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            run_async()
        g.replay()
        stream.synchronize()
        e0.record(stream)
        for _ in range(20):
            g.replay()
        e1.record(stream)
        e1.synchronize()
        ctx.check(L.setops_gpu_synchronize(ctx.handle))
        t_graph = e0.elapsed_time(e1) * 1e-3 / 20
        if int(dlen.item()) != int(n_out.value):
            raise SystemExit(f"k={k}: the graph replay gave {int(dlen.item())} results")
        reps = 20
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3 / reps
        nin = sum(int(x.size) for x in sets)
        alg = 4 * nin + 4 * int(n_out.value)
        core = int(0.05 * min(int(x.size) for x in sets))
        if int(n_out.value) < core:
            raise SystemExit(f"k={k}: {n_out.value} results, below the {core}-element core")
        import oracle
        want = oracle.svs_generic(sets)
        if not np.array_equal(out[:int(n_out.value)].cpu().numpy().view(np.uint32), want):
            raise SystemExit(f"k={k}: GPU result differs from svs_generic")
        cpu = cpu_kset_baseline(sets, want.size) if with_cpu else None
        # the small_adaptive path on the same sets (synchronous calls, like
        # ms_per_synchronous_call of SvS)
        n_ad = C.c_size_t()

        def run_ad():
            ctx.check(L.setops_gpu_adaptive(ctx.handle, ptrs, lens, k, out.data_ptr(),
                                            out.numel(), C.byref(n_ad), 0))
        run_ad()
        if n_ad.value != want.size or not np.array_equal(
                out[:want.size].cpu().numpy().view(np.uint32), want):
            raise SystemExit(f"k={k}: small_adaptive differs from svs_generic")
        e0.record(stream)
        for _ in range(reps):
            run_ad()
        e1.record(stream)
        e1.synchronize()
        t_ad = e0.elapsed_time(e1) * 1e-3 / reps
        rows.append({"k": k, "sizes": [int(x.size) for x in sets], "out": int(n_out.value),
                     "ms": 1e3 * t_dev, "kset_per_s": 1.0 / t_dev,
                     "GBps_algorithmic": alg / t_dev / 1e9, "frac_of_peak": alg / t_dev / 1e9 / peak,
                     "ms_per_synchronous_call": 1e3 * t, "ms_graph_replay": 1e3 * t_graph,
                     "GBps_graph_replay": alg / t_graph / 1e9,
                     "results_match_svs_generic": True,
                     "small_adaptive_ms_per_synchronous_call": 1e3 * t_ad,
                     "cpu_baseline": cpu})
    return {"workload": "k-set SvS: k in {3, 5, 8}, |S_i| = 2^22 / i, density 0.2, core 5 % of "
                        "the smallest set, u32, materialised, smallest first; inputs resident",
            "api": "setops_gpu_svs_async back to back, device pointers (ms); setops_gpu_svs, "
                   "which waits for its result length (ms_per_synchronous_call)",
            "rows": rows}


SERVE_SEED = 20240612


def cpu_serve_baseline(idx, ids, ks, plain_counts) -> dict:
    """The reference's CPU path answering the same query stream: svs_generic
    per query with each baseline as its 2-set function, queries spread over
    all cores (8,000 queries), and single-core on 500; the answers' lengths
    must equal the GPU's plain path's."""
    import oracle
    cores = oracle.host_cores()
    groups = [sorted((idx.list(int(i)) for i in ids[q][:ks[q]]), key=len)
              for q in range(min(8000, ks.size))]
    allc, single = {}, {}
    for algo in (oracle.SHUFFLING_W8, oracle.SIMD_GALLOPING_W16, oracle.BMISS_W4):
        t0 = time.perf_counter()
        c = oracle.run_svs_groups(groups, cores, algo=algo)
        allc[oracle.ALGO_NAMES[algo]] = len(groups) / (time.perf_counter() - t0)
        n = min(plain_counts.size, c.size)
        if not np.array_equal(c[:n], plain_counts[:n]):
            raise SystemExit("serving: CPU answers' lengths differ from the GPU's")
        t0 = time.perf_counter()
        oracle.run_svs_groups(groups[:500], 1, algo=algo)
        single[oracle.ALGO_NAMES[algo]] = 500 / (time.perf_counter() - t0)
    best = max(allc, key=allc.get)
    return {"value": allc[best], "unit": "queries/s", "cores": cores, "kind": "port",
            "best": best, "all_cores": allc,
            "single_core": {"value": max(single.values()), "cores": 1, "all": single,
                            "sample_queries": 500},
            "sample": f"the first {len(groups)} queries of the stream, spread over {cores} "
                      "threads (closed loop: throughput, no arrival process)",
            "arch": os.uname().machine}


def serve_leg(ctx, rates, with_cpu: bool = True) -> dict:
    """Served k-set queries (the reference's serving configuration): a
    resident index of 1,000,000 posting lists with rank-size Zipf(1.1)
    lengths clipped to [1, 2^20] over 2^26 documents; queries of k ~ U{2..6}
    lists drawn Zipf(1.1) over popularity, arriving as a Poisson stream at
    each rate (open loop: latency from scheduled arrival to completion).
    Beside it, the plain path: one setops_gpu_svs call per query."""
    import ctypes as C

    import torch

    import simd_set_operations_gb300 as so
    from simd_set_operations_gb300 import _lib, datasets as ds
    L = _lib.lib
    nl = 1_000_000
    idx = ds.gen_index(SERVE_SEED, nl, 1 << 20, 1.1, 1 << 26)
    nq_max = max(min(int(max(rates) * 1.0), 300_000), 20_000)
    ids, ks = ds.gen_queries(SERVE_SEED + 1, nq_max, nl, 2, 6, 1.1)
    out = {"workload": "1,000,000 posting lists, rank-size Zipf(1.1) lengths in [1, 2^20] "
                       f"({int(idx.pool.size)} postings, {4 * int(idx.pool.size) / 1e6:.1f} MB "
                       "resident) over 2^26 documents; queries k ~ U{2..6} lists, Zipf(1.1) "
                       "over popularity; Poisson arrivals; answers materialised",
           "rates": []}
    with so.Server(idx.pool, idx.offs, idx.lens, budget=512 << 20, ctx=ctx) as srv:
        srv.run_load(ids[:2000], ks[:2000], rate_qps=20000, seed=7)  # warm-up
        for rate in rates:
            nq = min(nq_max, max(int(rate * 1.0), 10_000))  # about a second of arrivals
            st0 = srv.stats()
            lat, cnt, el = srv.run_load(ids[:nq], ks[:nq], rate_qps=float(rate), seed=11)
            st1 = srv.stats()
            lat_ms = lat.astype(np.float64) * 1e-6
            out["rates"].append({
                "offered_qps": rate, "queries": nq, "achieved_qps": nq / el,
                "p50_ms": float(np.percentile(lat_ms, 50)),
                "p99_ms": float(np.percentile(lat_ms, 99)),
                "mean_answer": float(cnt.mean()),
                "batches": st1["batches"] - st0["batches"],
                "mean_batch": (st1["queries"] - st0["queries"]) / max(st1["batches"] - st0["batches"], 1),
            })
    # the plain path: one synchronous k-set call per query on device
    # pointers, looped in C
    pool = torch.from_numpy(idx.pool.view(np.int32)).cuda()
    dout = torch.empty(1 << 20, dtype=torch.int32, device="cuda")
    nplain = 2000
    lat = np.zeros(nplain, np.uint64)
    cnt = np.zeros(nplain, np.uint64)
    secs = C.c_double()

    def plain(nq):
        ctx.check(L.setops_bench_queries_one_by_one(
            ctx.handle, pool.data_ptr(), idx.offs.ctypes.data, idx.lens.ctypes.data,
            ids.ctypes.data, ks.ctypes.data, ids.shape[1], nq, dout.data_ptr(), dout.numel(),
            lat.ctypes.data, cnt.ctypes.data, C.byref(secs)))
        return secs.value
    plain(50)
    el = plain(nplain)
    tt = lat.astype(np.float64) * 1e-6
    out["plain_one_call_per_query"] = {
        "api": "setops_gpu_svs per query on device pointers, sequential, looped in C "
               "(setops_bench_queries_one_by_one)", "queries": nplain,
        "qps": nplain / el, "p50_ms": float(np.percentile(tt, 50)),
        "p99_ms": float(np.percentile(tt, 99))}
    if with_cpu:
        out["cpu_baseline"] = cpu_serve_baseline(idx, ids, ks, cnt)
    best = max(r["achieved_qps"] for r in out["rates"])
    out["best_served_qps"] = best
    out["speedup_vs_plain"] = best / out["plain_one_call_per_query"]["qps"]
    return out


def summarize(roofline, e2e, cpu, config0, batch, kset, serve) -> dict:
    """The figures of every leg in a few keys, placed early in the line."""
    g = lambda d, *ks: None if d is None else (  # noqa: E731
        g(d.get(ks[0]), *ks[1:]) if len(ks) > 1 else d.get(ks[0]))
    r = lambda x, n=3: None if x is None else round(float(x), n)  # noqa: E731
    out = {"headline_frac": r(g(roofline, "frac")),
           "sweep_e2e_pairs_per_s": r(g(e2e, "value"), 1),
           "sweep_e2e_per_call_pairs_per_s": r(g(e2e, "per_call", "value"), 1),
           "sweep_cpu_pairs_per_s": r(g(cpu, "value"), 1)}
    if config0:
        out["config0"] = {"pairs_per_s": r(config0["pairs_per_s"], 1),
                          "frac": r(config0["frac_of_peak"]),
                          "e2e_pairs_per_s": r(g(config0, "e2e", "pairs_per_s"), 1),
                          "cpu_pairs_per_s": r(g(config0, "cpu_baseline", "value"), 1)}
    if batch:
        out["batch"] = {"pairs_per_s": r(batch["pairs_per_s"], 0),
                        "frac": r(batch["frac_of_peak"]),
                        "x_one_launch_per_pair": r(batch["speedup_vs_one_launch_per_pair"], 1),
                        "cpu_pairs_per_s": r(g(batch, "cpu_baseline", "value"), 0),
                        "bsr_pairs_per_s": r(g(batch, "bsr_subset", "pairs_per_s"), 0),
                        "bsr_frac": r(g(batch, "bsr_subset", "frac_of_peak")),
                        "bsr_x_one_call_per_pair":
                            r(g(batch, "bsr_subset", "speedup_vs_one_call_per_pair"), 1),
                        "bsr_cpu_pairs_per_s": r(g(batch, "bsr_subset", "cpu_baseline", "value"), 0)}
    if kset:
        out["kset"] = [{"k": row["k"], "ms": r(row["ms"], 4), "frac": r(row["frac_of_peak"]),
                        "cpu_per_s": r(g(row, "cpu_baseline", "value"), 2)}
                       for row in kset["rows"]]
    if serve:
        out["serve"] = {"best_qps": r(serve["best_served_qps"], 0),
                        "x_plain": r(serve["speedup_vs_plain"], 1),
                        "p99_ms": {str(x["offered_qps"]): r(x["p99_ms"]) for x in serve["rates"]},
                        "cpu_qps": r(g(serve, "cpu_baseline", "value"), 0)}
    return out


KERNEL_NAMES = {
    "bitmap/0": "window_kernel (bitmap tiles, B in register windows)",
    "bitmap/7": "window_kernel, coarse bitmaps for sparse tiles",
    "bitmap/8": "awindow_kernel (bitmap tiles, A tiles and B windows staged in shared memory "
                "by cp.async)",
}


def run_gb300(args):
    import ctypes as C

    import torch

    import simd_set_operations_gb300 as so
    from simd_set_operations_gb300 import _lib

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    ctx = so.Context(local)
    # a dedicated stream, current for torch too, so that CUDA events and the
    # library's kernels are ordered on the same stream
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream)
    L = _lib.lib

    # the array policy, tuned on this GPU before anything is timed (bands up
    # to 2^16 : 1, test pairs of up to 2^25 elements, the sweep's density)
    policy = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        tab = so.autotune(band_lo=0, band_hi=16, max_elems=1 << 25, density=DENSITY, reps=3,
                          bsr=False, ctx=ctx)
        policy = {"tuned_cells": tab["tuned_cells"], "seconds": time.perf_counter() - t0,
                  "device": tab["key"]["device"],
                  "table": {cell: so.describe_flags(f) for cell, f in tab["cells"].items()},
                  "note": "cell 'band,class': size ratio in [2^band, 2^(band+1)), smaller "
                          "input < 2^12 / 2^16 / 2^22 / above (class 0-3)"}

    sel = [int(x) for x in args.pairs.split(",")]
    pairs = [p for i, p in enumerate(make_sweep(rank)) if i in sel]
    dev = []
    for s, l in pairs:
        ds_ = torch.from_numpy(s.view(np.int32)).cuda()
        dl_ = torch.from_numpy(l.view(np.int32)).cuda()
        out = torch.empty(s.size, dtype=torch.int32, device="cuda")
        dev.append((ds_, dl_, out))
    lens = torch.zeros(len(pairs), dtype=torch.int64, device="cuda")
    h = ctx.handle

    # the headline kernel: the 2^24 x 2^24 pair (size ratio 1 -> tiled bitmap)
    head = max(range(len(pairs)), key=lambda i: pairs[i][0].size)

    def launch(i):
        (s, l), (ds_, dl_, out) = pairs[i], dev[i]
        rc = L.setops_gpu_intersect_async(h, ds_.data_ptr(), s.size, dl_.data_ptr(), l.size,
                                          out.data_ptr(), s.size, lens.data_ptr() + 8 * i, 0)
        if rc != 0:
            ctx.check(rc)

    def step(ev=None, rec=None):
        # ev: an event pair around the headline launch (every event recorded
        # between launches costs device time, so only that one is bracketed);
        # rec: how to record an event (inside a graph capture: an external
        # record, so that the event times every replay)
        for i in range(len(pairs)):
            if ev is not None and i == head:
                rec(ev[0]) if rec else ev[0].record(stream)
            launch(i)
            if ev is not None and i == head:
                rec(ev[1]) if rec else ev[1].record(stream)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # warmup (at least W steps and about 2 s of load for the clock sampler)
    sampler = ClockSampler(local)
    sampler.start()
    t_w = time.perf_counter()
    nw = 0
    while nw < args.warmup or time.perf_counter() - t_w < args.min_warmup_seconds:
        step()
        nw += 1
        if nw % 50 == 0:
            torch.cuda.synchronize()
    torch.cuda.synchronize()
    ctx.synchronize()

    # exactness of the step's results (counts are known from generation)
    got = lens.cpu().tolist()
    want = [int(SELECTIVITY * s.size) for s, _ in pairs]
    if got != want:
        raise SystemExit(f"wrong intersection sizes {got} != {want}")

    # timed region: K steps, no host synchronisation inside; one event pair
    # around the headline launch of each step (on the launching stream)
    def mk():
        return torch.cuda.Event(enable_timing=True)
    evs = [(mk(), mk()) for _ in range(args.steps)]
    for e0, e1 in evs:  # creates the events before any capture
        e0.record(stream)
        e1.record(stream)
    graph = None
    launches0 = ctx.launch_count
    if not args.no_graph:
        # the K steps captured once into a CUDA graph (the library's
        # asynchronous calls: the steady-state form of a repeated workload);
        # one replay is the timed region
        def rec(e):
            ctx.check(L.setops_bench_record_event(C.c_void_p(e.cuda_event),
                                                  C.c_void_p(stream.cuda_stream)))
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            for k in range(args.steps):
                step(evs[k], rec)
        launches = ctx.launch_count - launches0
        graph.replay()  # untimed
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    t_start, t_end = mk(), mk()
    t_start.record(stream)
    if graph is not None:
        graph.replay()
    else:
        for k in range(args.steps):
            step(evs[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    if graph is None:
        launches = ctx.launch_count - launches0
    # the same K steps as plain calls, for comparison (no events inside)
    p0, p1 = mk(), mk()
    p0.record(stream)
    for k in range(args.steps):
        step()
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1) / args.steps
    clocks = sampler.stop()
    head_times = [e0.elapsed_time(e1) for e0, e1 in evs]
    wall_ms = t_start.elapsed_time(t_end)
    el_s = max_over_ranks(wall_ms / 1e3)
    value = job_value(world, len(pairs), args.steps, el_s)

    # per-pair kernel times, outside the timed region: each pair launched 20
    # times back to back between one event pair
    per_pair = []
    for i in range(len(pairs)):
        ts = []
        for _ in range(3):
            e0, e1 = mk(), mk()
            e0.record(stream)
            for _ in range(20):
                launch(i)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 20)
        per_pair.append(ts)

    # roofline: the headline kernel, from its events inside the timed region
    s_h, l_h = pairs[head]
    nout = int(SELECTIVITY * s_h.size)
    head_ms = statistics.mean(head_times)
    algo_bytes = algorithmic_bytes(s_h.size, l_h.size, nout)
    achieved = algo_bytes / (head_ms / 1e3) / 1e9
    peak, peak_kind = read_peak()
    traffic = read_traffic()
    head_flags = ctx.get_policy_class(False, 0, 3)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": f"{KERNEL_NAMES.get(so.describe_flags(head_flags), so.describe_flags(head_flags))}"
                          " (2^24 x 2^24 pair, materialise)",
                "algorithmic_bytes_per_launch": algo_bytes,
                "launch_ms_mean": head_ms, "peak_source": f"{peak_kind} (hbm_gbs)"}
    sweep = []
    for (s, l), p in zip(pairs, per_pair):
        n = int(SELECTIVITY * s.size)
        ms = statistics.mean(p)
        row = {"small": int(s.size), "large": int(l.size), "out": n,
               "ms_back_to_back": ms, "ms_min": min(p),
               "GBps_algorithmic": algorithmic_bytes(s.size, l.size, n) / (ms / 1e3) / 1e9}
        if l.size >= 32 * s.size:  # search band: the sectors the probes touch
            tb = touched_bytes(s.size, l.size, n)
            row["touched_bytes_est"] = tb
            row["GBps_touched_est"] = tb / (ms / 1e3) / 1e9
        sweep.append(row)

    # e2e through the host-pointer C ABI
    e2e = None
    if not args.no_e2e:
        pinned = []
        for s, l in pairs:
            ps = torch.from_numpy(s.view(np.int32)).pin_memory().numpy().view(np.uint32)
            pl = torch.from_numpy(l.view(np.int32)).pin_memory().numpy().view(np.uint32)
            po = torch.empty(s.size, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
            pinned.append((ps, pl, po))
        n_out = C.c_size_t()

        def step_e2e():
            tot_out = 0
            for ps, pl, po in pinned:
                rc = L.setops_gpu_intersect(h, ps.ctypes.data, ps.size, pl.ctypes.data, pl.size,
                                            po.ctypes.data, ps.size, C.byref(n_out), _lib.HOST)
                if rc != 0:
                    ctx.check(rc)
                tot_out += n_out.value
            return tot_out

        # the whole step in one call: setops_gpu_intersect_pairs overlaps the
        # balanced pair's input copy with the in-place searches
        npr = len(pinned)
        P, S = C.c_void_p * npr, C.c_size_t * npr
        outs2 = [torch.empty(ps.size, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
                 for ps, _, _ in pinned]
        arr_a, arr_la = P(*[ps.ctypes.data for ps, _, _ in pinned]), S(*[ps.size for ps, _, _ in pinned])
        arr_b, arr_lb = P(*[pl.ctypes.data for _, pl, _ in pinned]), S(*[pl.size for _, pl, _ in pinned])
        arr_o, arr_co = P(*[o.ctypes.data for o in outs2]), S(*[o.size for o in outs2])
        arr_len = S()

        def step_e2e_pairs():
            rc = L.setops_gpu_intersect_pairs(h, npr, arr_a, arr_la, arr_b, arr_lb, arr_o, arr_co,
                                              arr_len, _lib.HOST)
            if rc != 0:
                ctx.check(rc)
            return sum(int(x) for x in arr_len)

        def timed(fn, steps):
            barrier()
            t0 = time.perf_counter()
            tot = 0
            for _ in range(steps):
                tot = fn()
            el = time.perf_counter() - t0
            barrier()
            return max_over_ranks(el), tot

        for _ in range(max(2, args.warmup // 2)):
            step_e2e()
            step_e2e_pairs()
        e2e_steps = max(3, min(args.steps, 20))
        pc_el, tot_out = timed(step_e2e, e2e_steps)
        e_el, tot_out2 = timed(step_e2e_pairs, e2e_steps)
        same = tot_out2 == tot_out and all(
            int(arr_len[i]) <= po.size and np.array_equal(outs2[i][:int(arr_len[i])], po[:int(arr_len[i])])
            for i, (_, _, po) in enumerate(pinned))
        h2d = sum(4 * (s.size + l.size) for s, l in pairs)
        d2h = 4 * tot_out + 8 * len(pairs)
        # what crosses the host link: a search-band pair is read in place and
        # moves only the sectors its probes touch; a balanced pair is copied
        moved = 0
        for s, l in pairs:
            moved += touched_bytes(s.size, l.size, int(SELECTIVITY * s.size)) \
                if l.size >= 32 * s.size else 4 * (s.size + l.size)
        e2e = {"value": job_value(world, len(pairs), e2e_steps, e_el), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
               "ms_per_step": 1e3 * e_el / e2e_steps,
               "h2d_bytes_moved_est": moved,
               "api": "setops_gpu_intersect_pairs(..., SETOPS_HOST), one call per step from "
                      "pinned host buffers: the search-band pairs are read in place over the host "
                      "link (NVLink-C2C) on a second stream while the balanced pair's inputs are "
                      "copied; results written into the pinned outputs",
               "results_match_per_call": bool(same),
               "per_call": {"value": job_value(world, len(pairs), e2e_steps, pc_el), "unit": UNIT,
                            "ms_per_step": 1e3 * pc_el / e2e_steps,
                            "api": "setops_gpu_intersect(..., SETOPS_HOST), one call per pair, "
                                   "the same buffers: each pair's copies and kernel in turn"}}

    # CPU baseline (rank 0 at N=1 only), also the cross-check of the results
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and len(pairs) == len(SMALL_EXPS):
        import oracle
        cores = oracle.host_cores()
        v1, s1, detail, counts, outs, spent = cpu_sweep_best(pairs, 1, args.cpu_sample_seconds)
        vall, sall, _, _, _, spent2 = cpu_sweep_best(pairs, min(cores, len(pairs)), 2.0)
        for i, ((s, l), (ds_, dl_, out)) in enumerate(zip(pairs, dev)):
            n = int(lens[i])
            g = out[:n].cpu().numpy().view(np.uint32)
            if n != counts[i] or not np.array_equal(g, outs[i][:n]):
                raise SystemExit(f"GPU result of pair {i} differs from the CPU path")
        cpu = {"value": vall, "unit": UNIT, "cores": min(cores, len(pairs)), "kind": "port",
               "sample": "the 4-pair sweep; each baseline timed per pair, best per pair kept; "
                         "all-cores = pairs spread over threads (one pair never spans threads)",
               "single_core": {"value": v1, "cores": 1, "sweep_seconds": s1},
               "algorithms": detail, "cpu_seconds_spent": spent + spent2,
               "host_cores": cores, "arch": os.uname().machine,
               "results_match_gpu": True}

    config0 = None
    if rank == 0 and not args.no_config0:
        config0 = config0_leg(ctx, stream, min(args.cpu_sample_seconds, 6.0),
                              with_cpu=not args.no_cpu_baseline)
    batch = None
    if rank == 0 and not args.no_batch:
        batch = batch_leg(ctx, stream, args.batch_pairs)
        batch["bsr_subset"] = batch_bsr_leg(ctx, stream, args.bsr_pairs)
    kset = None
    if rank == 0 and not args.no_kset:
        kset = kset_leg(ctx, stream, ks=tuple(int(x) for x in args.kset_ks.split(",")),
                        with_cpu=not args.no_cpu_baseline)
    serve = None
    if rank == 0 and not args.no_serve:
        serve = serve_leg(ctx, [int(x) for x in args.serve_rates.split(",")],
                          with_cpu=not args.no_cpu_baseline)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT,
        "summary": summarize(roofline, e2e, cpu, config0, batch, kset, serve),
        "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded; reference generator shape)",
        "config": workload_config(sel),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": int(launches), "clocks": clocks, "policy": policy, "sweep": sweep,
        "config0": config0,
        "batch": batch, "kset": kset, "serve": serve,
        "timing": {"bracket_ms_total": wall_ms, "headline_ms_total": sum(head_times),
                   "cuda_graph": graph is not None,
                   "plain_calls_ms_per_step": plain_ms,
                   "note": "value = pairs / CUDA-event time of the K-step bracket: one replay "
                           "of a CUDA graph holding the K steps' asynchronous library calls "
                           "(--no-graph: the calls themselves), one event pair per step "
                           "around the headline launch (external event records inside the "
                           "graph); plain_calls_ms_per_step: the same K steps as plain calls "
                           "after it; sweep[].ms_back_to_back: each pair launched 20 times "
                           "back to back"},
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
