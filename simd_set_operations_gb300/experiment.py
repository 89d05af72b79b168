"""Experiment files, dataset generation, a timer registry and a runner for
this library's GPU algorithms, in the reference benchmark's formats, so that
its experiment files, dataset directories and results readers carry over.

The reference's pieces and what stands in for them here:

* experiment file (benchmark/src/schema.rs:13-84): TOML with
  ``[algorithm_sets]``, ``[[experiment]]`` (name, title, dataset,
  ``algorithms`` or ``algorithm_set``, ``relative_to``) and ``[[dataset]]``
  (synthetic: vary, to, step, gen_count, set_count, density, selectivity,
  max_len, skewness_factor -- percentages in thousandths, max_len as log2);
* ``xvalues`` / ``props_at_x`` (benchmark/src/lib.rs:27-58);
* dataset generation (benchmark/src/bin/generate.rs:115-240): one datafile
  per (x, i) at ``<datasets>/<name>/<x>/<i>``, 2-set or k-set by set_count,
  from this library's seeded generators (the reference's are unseeded);
* the timer registry (benchmark/src/timer.rs:75-259): names -> algorithms.
  Registered here: the GPU algorithms, ``gpu_auto``, ``gpu_merge``,
  ``gpu_galloping``, ``gpu_bitmap``, ``gpu_bitmap_coarse`` (the tiled bitmap
  kernel with coarse bitmaps for sparse tiles) (2-set; on k-set data:
  smallest-first SvS with that kernel), ``gpu_svs`` (k-set, automatic),
  ``gpu_small_adaptive`` (k-set, small_adaptive), ``gpu_bsr`` (BSR
  2-set; encoding outside the timed region, as the reference's harness,
  benchmark/src/timer/harness.rs:121-122).  Names of the reference's CPU
  algorithms are reported as unknown, as the reference does for names it
  cannot run;
* the runner (benchmark/src/bin/benchmark.rs:57-250) and ``results.json``
  (schema.rs:86-130): per dataset, per algorithm, one ``ResultRun`` per x
  with one time per datafile in nanoseconds.  Times are CUDA-event times of
  one call on device-resident inputs after a time-based warm-up; the CPU
  counter fields (cache, branches, cycles) are null.

Run: ``python -m simd_set_operations_gb300.experiment generate|run
--experiment FILE --datasets DIR [--out results.json] [--count-only]
[experiment names ...]``.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import sys
import time
import tomllib
import zlib
from dataclasses import dataclass
from pathlib import Path
from typing import Callable

import numpy as np

PERCENT = 1000  # schema.rs:10: an integer i stands for i / 1000


# ---------------------------------------------------------------------------
# experiment file

def load_experiment(path) -> dict:
    with open(path, "rb") as f:
        exp = tomllib.load(f)
    exp.setdefault("experiment", [])
    exp.setdefault("dataset", [])
    exp.setdefault("algorithm_sets", {})
    return exp


def experiment_algorithms(exp: dict, entry: dict) -> list[str]:
    """get_algorithms (benchmark/src/lib.rs:60-69)."""
    if "algorithms" in entry:
        return list(entry["algorithms"])
    name = entry.get("algorithm_set")
    if name not in exp["algorithm_sets"]:
        raise ValueError(f"algorithm set {name} not found")
    return list(exp["algorithm_sets"][name])


_VARY = {"selectivity": "selectivity", "density": "density", "size": "max_len",
         "skew": "skewness_factor", "set_count": "set_count"}


def xvalues(info: dict) -> range:
    """xvalues (benchmark/src/lib.rs:27-44): from the varied property's value
    to `to`, by `step`."""
    if info["type"] == "real":
        return range(info["set_count_start"], info["set_count_end"] + 1)
    return range(int(info[_VARY[info["vary"]]]), int(info["to"]) + 1, int(info["step"]))


def props_at_x(info: dict, x: int) -> dict:
    """props_at_x (benchmark/src/lib.rs:46-58)."""
    props = {k: int(info[k]) for k in ("set_count", "density", "selectivity", "max_len",
                                       "skewness_factor")}
    props[_VARY[info["vary"]]] = int(x)
    return props


def _skew(set_index: int, skew_factor: int) -> int:
    # get_skew (benchmark/src/generators.rs:220-224): (index + 1)^(factor / 1000)
    return max(int(float(set_index + 1) ** (skew_factor / PERCENT)), 1)


def generate_sets(props: dict, seed: int) -> list[np.ndarray]:
    """One synthetic intersection (generate_synthetic_intersection,
    benchmark/src/bin/generate.rs:223-234): two sets, the smaller 2^max_len /
    2^(skew/1000) long, or a k-set group, smallest first."""
    from . import datasets as ds
    dens, sel = props["density"] / PERCENT, props["selectivity"] / PERCENT
    large = 1 << props["max_len"]
    if props["set_count"] == 2:
        small = large // _skew(1, props["skewness_factor"])
        s, l = ds.gen_twoset(seed, dens, sel, small, large)
        return [s, l]
    return ds.gen_kset(seed, dens, sel, large, props["skewness_factor"] / PERCENT,
                       props["set_count"])


def _seed(name: str, x: int, i: int) -> int:
    return zlib.crc32(f"{name}/{x}/{i}".encode()) * 1_000_003 + 17


def generate(exp: dict, datasets_dir, names: list[str] | None = None) -> list[Path]:
    """Writes every synthetic dataset of the experiment file (or those named):
    <datasets_dir>/<name>/<x>/<i> datafiles and <name>.json (the dataset's
    description, as the reference's generator writes it)."""
    from . import datasets as ds
    out = []
    root = Path(datasets_dir)
    for info in exp["dataset"]:
        if names and info["name"] not in names:
            continue
        if info.get("type") != "synthetic":
            raise ValueError(f"dataset {info['name']}: only synthetic datasets are generated here")
        (root / info["name"]).mkdir(parents=True, exist_ok=True)
        (root / (info["name"] + ".json")).write_text(json.dumps(info, indent=2))
        for x in xvalues(info):
            xdir = root / info["name"] / str(x)
            xdir.mkdir(parents=True, exist_ok=True)
            props = props_at_x(info, x)
            for i in range(int(info["gen_count"])):
                p = xdir / str(i)
                ds.datafile_write(p, generate_sets(props, _seed(info["name"], x, i)))
                out.append(p)
    return out


# ---------------------------------------------------------------------------
# timer registry

@dataclass
class Timer:
    """A registered algorithm: `time(ctx, sets, count_only, warmup_s)`
    returns the nanoseconds of one call on device-resident inputs."""
    name: str
    time: Callable


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _timed(ctx, call, warmup_s: float) -> int:
    """Time-based warm-up (at least one call), then one call between CUDA
    events on the context's stream (harness.rs:35-97 times one run too)."""
    import torch
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    call()
    while time.perf_counter() - t0 < warmup_s:
        call()
    ctx.synchronize()
    e0, e1 = _events()
    e0.record(stream)
    call()
    e1.record(stream)
    e1.synchronize()
    ctx.synchronize()
    return int(e0.elapsed_time(e1) * 1e6)


def _pair_timer(algo: int):
    def run(ctx, sets, count_only, warmup_s):
        import torch

        from ._lib import lib
        from . import ALGO_AUTO
        if len(sets) > 2:  # k-set data: smallest-first SvS with this kernel
            return _svs_timer(algo)(ctx, sets, count_only, warmup_s)
        a, b = sets
        da = torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
        db = torch.from_numpy(np.ascontiguousarray(b).view(np.int32)).cuda()
        cap = min(a.size, b.size)
        out = None if count_only else torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
        ln = torch.zeros(1, dtype=torch.int64, device="cuda")

        def call():
            ctx.check(lib.setops_gpu_intersect_async(
                ctx.handle, da.data_ptr(), a.size, db.data_ptr(), b.size,
                None if out is None else out.data_ptr(), 0 if out is None else cap,
                ln.data_ptr(), algo if algo is not None else ALGO_AUTO))
        return _timed(ctx, call, warmup_s)
    return run


def _svs_timer(algo: int | None):
    def run(ctx, sets, count_only, warmup_s):
        import torch

        from ._lib import lib
        from . import ALGO_AUTO
        dsets = [torch.from_numpy(np.ascontiguousarray(s).view(np.int32)).cuda() for s in sets]
        k = len(sets)
        ptrs = (C.c_void_p * k)(*[d.data_ptr() for d in dsets])
        lens = (C.c_size_t * k)(*[int(s.size) for s in sets])
        cap = min(int(s.size) for s in sets)
        out = None if count_only else torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
        ln = torch.zeros(1, dtype=torch.int64, device="cuda")

        def call():
            ctx.check(lib.setops_gpu_svs_async(
                ctx.handle, ptrs, lens, k, None if out is None else out.data_ptr(),
                0 if out is None else cap, ln.data_ptr(), algo if algo is not None else ALGO_AUTO))
        return _timed(ctx, call, warmup_s)
    return run


def _bsr_timer(ctx, sets, count_only, warmup_s):
    import torch

    from ._lib import lib
    if len(sets) != 2:
        raise ValueError("gpu_bsr takes 2-set data")
    enc = []
    for s in sets:  # encoding outside the timed region (harness.rs:121-122)
        d = torch.from_numpy(np.ascontiguousarray(s).view(np.int32)).cuda()
        bases = torch.empty(max(s.size, 1), dtype=torch.int32, device="cuda")
        states = torch.empty_like(bases)
        nw = C.c_size_t()
        ctx.check(lib.setops_gpu_bsr_from_sorted(ctx.handle, d.data_ptr(), s.size,
                                                 bases.data_ptr(), states.data_ptr(),
                                                 C.byref(nw), 0))
        enc.append((bases, states, int(nw.value)))
    (ba, sa, na), (bb, sb, nb) = enc
    cap = min(na, nb)
    ob = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    os_ = torch.empty_like(ob)
    n = C.c_size_t()
    cnt = C.c_uint64()

    def call():
        if count_only:
            ctx.check(lib.setops_gpu_intersect_bsr_count(
                ctx.handle, ba.data_ptr(), sa.data_ptr(), na, bb.data_ptr(), sb.data_ptr(), nb,
                C.byref(cnt), 0))
        else:
            ctx.check(lib.setops_gpu_intersect_bsr(
                ctx.handle, ba.data_ptr(), sa.data_ptr(), na, bb.data_ptr(), sb.data_ptr(), nb,
                ob.data_ptr(), os_.data_ptr(), cap, C.byref(n), 0))
    return _timed(ctx, call, warmup_s)


def _adaptive_timer(ctx, sets, count_only, warmup_s):
    """small_adaptive (setops/src/intersect/adaptive.rs:107-148) on the GPU:
    each call waits for its result length (the k-set entry point is
    synchronous)."""
    import torch

    from ._lib import lib
    if len(sets) < 2:
        raise ValueError("gpu_small_adaptive takes k-set data")
    dsets = [torch.from_numpy(np.ascontiguousarray(s).view(np.int32)).cuda() for s in sets]
    k = len(sets)
    ptrs = (C.c_void_p * k)(*[d.data_ptr() for d in dsets])
    lens = (C.c_size_t * k)(*[int(s.size) for s in sets])
    cap = min(int(s.size) for s in sets)
    out = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    n = C.c_size_t()
    cnt = C.c_uint64()

    def call():
        if count_only:
            ctx.check(lib.setops_gpu_adaptive_count(ctx.handle, ptrs, lens, k, C.byref(cnt), 0))
        else:
            ctx.check(lib.setops_gpu_adaptive(ctx.handle, ptrs, lens, k, out.data_ptr(), cap,
                                              C.byref(n), 0))
    return _timed(ctx, call, warmup_s)


# SETOPS_ALGO_BITMAP variant with coarse bitmaps for sparse tiles
BITMAP_COARSE_VARIANT = 7


def _registry() -> dict[str, Timer]:
    from . import ALGO_BITMAP, ALGO_GALLOP, ALGO_MERGE, VARIANT
    return {
        "gpu_auto": Timer("gpu_auto", _pair_timer(None)),
        "gpu_merge": Timer("gpu_merge", _pair_timer(ALGO_MERGE)),
        "gpu_galloping": Timer("gpu_galloping", _pair_timer(ALGO_GALLOP)),
        "gpu_bitmap": Timer("gpu_bitmap", _pair_timer(ALGO_BITMAP)),
        "gpu_bitmap_coarse": Timer("gpu_bitmap_coarse",
                                   _pair_timer(ALGO_BITMAP | VARIANT(BITMAP_COARSE_VARIANT))),
        "gpu_svs": Timer("gpu_svs", _svs_timer(None)),
        "gpu_bsr": Timer("gpu_bsr", _bsr_timer),
        "gpu_small_adaptive": Timer("gpu_small_adaptive", _adaptive_timer),
    }


TIMER_NAMES = ("gpu_auto", "gpu_merge", "gpu_galloping", "gpu_bitmap", "gpu_bitmap_coarse",
               "gpu_svs", "gpu_bsr", "gpu_small_adaptive")


def timer(name: str) -> Timer | None:
    """Timer::new (benchmark/src/timer.rs:24-36): None for an unknown name."""
    return _registry().get(name)


# ---------------------------------------------------------------------------
# runner

def _empty_run(x: int) -> dict:
    cache = {"rd_access": None, "rd_miss": None, "wr_access": None, "wr_miss": None}
    return {"x": int(x), "times": [], "l1d": dict(cache), "l1i": dict(cache), "ll": dict(cache),
            "branches": None, "branch_misses": None, "cpu_stalled_front": None,
            "cpu_stalled_back": None, "instructions": None, "cpu_cycles": None,
            "cpu_cycles_ref": None}


def run(exp: dict, datasets_dir, experiments: list[str] | None = None, count_only: bool = False,
        warmup_s: float = 0.05, ctx=None, timers: dict | None = None, log=print) -> dict:
    """run_experiments (benchmark/src/bin/benchmark.rs:94-200): every
    (dataset, algorithm) pair the chosen experiments need is run once over
    every datafile of every x.  Returns the results document."""
    from . import datasets as ds
    registry = timers if timers is not None else _registry()
    chosen = [e for e in exp["experiment"] if not experiments or e["name"] in experiments]
    need: dict[str, set] = {}
    for e in chosen:
        need.setdefault(e["dataset"], set()).update(experiment_algorithms(exp, e))
    if not need:
        raise ValueError("no algorithm matches found")
    if ctx is None and timers is None:
        from . import default_context
        ctx = default_context()
    if timers is None:
        # one stream for the library's launches and the timing events
        import torch
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        ctx.set_stream(stream)
    results = {}
    for info in exp["dataset"]:
        algos = need.get(info["name"])
        if not algos:
            continue
        log(info["name"])
        algo_results = {a: [] for a in sorted(algos)}
        for x in xvalues(info):
            xdir = Path(datasets_dir) / info["name"] / str(x)
            files = sorted(xdir.iterdir(), key=lambda p: (len(p.name), p.name))
            groups = [ds.datafile_read(f) for f in files]
            for name, runs in algo_results.items():
                t = registry.get(name)
                if t is None:
                    log(f"  unknown algorithm {name}")
                    continue
                rr = _empty_run(x)
                for sets in groups:
                    rr["times"].append(int(t.time(ctx, sets, count_only,
                                                  warmup_s / max(len(groups), 1))))
                runs.append(rr)
        results[info["name"]] = {"info": info, "algos": algo_results}
    return {"experiments": chosen, "datasets": results, "algorithm_sets": exp["algorithm_sets"]}


def main(argv=None) -> int:
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("command", choices=["generate", "run"])
    p.add_argument("--experiment", default="experiment.toml")
    p.add_argument("--datasets", default="datasets/")
    p.add_argument("--out", default="results.json")
    p.add_argument("--count-only", action="store_true")
    p.add_argument("--warmup-seconds", type=float, default=0.05)
    p.add_argument("names", nargs="*", help="datasets (generate) or experiments (run)")
    a = p.parse_args(argv)
    exp = load_experiment(a.experiment)
    if a.command == "generate":
        n = len(generate(exp, a.datasets, a.names or None))
        print(f"{n} datafiles written under {a.datasets}")
        return 0
    res = run(exp, a.datasets, a.names or None, a.count_only, a.warmup_seconds)
    Path(a.out).write_text(json.dumps(res))
    print(f"results written to {a.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
