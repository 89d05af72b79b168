"""The experiment runner (simd_set_operations_gb300/experiment.py): the
reference benchmark's experiment file, x values and dataset layout
(benchmark/src/lib.rs:27-58, benchmark/src/bin/generate.rs:115-240) and its
results document (benchmark/src/schema.rs:86-130).  CPU: parsing, generation
and the results layout with a stand-in timer; GPU: the registered timers."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from simd_set_operations_gb300 import datasets as ds
from simd_set_operations_gb300 import experiment as ex

PKG = Path(__file__).resolve().parents[1] / "simd_set_operations_gb300"

SMALL = """
[algorithm_sets]
two = ["gpu_auto", "gpu_merge", "not_a_gpu_algorithm"]

[[experiment]]
name = "e2"
title = "2-set"
dataset = "d2"
relative_to = "gpu_merge"
algorithm_set = "two"

[[experiment]]
name = "ek"
title = "k-set"
dataset = "dk"
algorithms = ["gpu_svs"]

[[dataset]]
name = "d2"
type = "synthetic"
set_count = 2
gen_count = 2
vary = "size"
max_len = 8
to = 12
step = 2
selectivity = 100
skewness_factor = 1000
density = 300

[[dataset]]
name = "dk"
type = "synthetic"
set_count = 3
gen_count = 2
vary = "set_count"
to = 4
step = 1
selectivity = 100
skewness_factor = 1000
density = 200
max_len = 10
"""


@pytest.fixture()
def small(tmp_path):
    f = tmp_path / "exp.toml"
    f.write_text(SMALL)
    return ex.load_experiment(f), tmp_path / "datasets"


def test_example_file_parses():
    exp = ex.load_experiment(PKG / "experiment_gpu.toml")
    names = {d["name"] for d in exp["dataset"]}
    for e in exp["experiment"]:
        assert e["dataset"] in names
        for a in ex.experiment_algorithms(exp, e):
            assert a in ex.TIMER_NAMES


def test_xvalues_and_props(small):
    exp, _ = small
    d2, dk = exp["dataset"]
    assert list(ex.xvalues(d2)) == [8, 10, 12]
    assert ex.props_at_x(d2, 10)["max_len"] == 10 and ex.props_at_x(d2, 10)["density"] == 300
    assert list(ex.xvalues(dk)) == [3, 4]
    assert ex.props_at_x(dk, 4)["set_count"] == 4


def test_generate_layout_and_contents(small):
    exp, root = small
    files = ex.generate(exp, root)
    assert len(files) == 3 * 2 + 2 * 2
    assert json.loads((root / "d2.json").read_text())["name"] == "d2"
    # 2-set at x = 10: |large| = 2^10, |small| = 2^10 / 2^(1000/1000) = 512
    a, b = ds.datafile_read(root / "d2" / "10" / "1")
    assert (a.size, b.size) == (512, 1024)
    assert np.all(np.diff(a.astype(np.int64)) > 0) and np.all(np.diff(b.astype(np.int64)) > 0)
    # k-set at x = 4: four sets, smallest first, 2^10 / (i+1)
    ks = ds.datafile_read(root / "dk" / "4" / "0")
    assert [s.size for s in ks] == [256, 341, 512, 1024]
    # generation is seeded: the same file twice
    again = ex.generate(exp, root, ["dk"])
    assert all(np.array_equal(x, y) for x, y in zip(ks, ds.datafile_read(root / "dk" / "4" / "0")))
    assert len(again) == 4


def test_results_layout_with_a_stand_in_timer(small):
    exp, root = small
    ex.generate(exp, root)
    seen = []
    fake = {n: ex.Timer(n, lambda ctx, sets, co, w, n=n: seen.append((n, len(sets))) or 123)
            for n in ("gpu_auto", "gpu_merge", "gpu_svs")}
    logs = []
    res = ex.run(exp, root, timers=fake, log=logs.append)
    assert [e["name"] for e in res["experiments"]] == ["e2", "ek"]
    assert set(res["datasets"]) == {"d2", "dk"}
    d2 = res["datasets"]["d2"]
    assert d2["info"]["name"] == "d2"
    assert set(d2["algos"]) == {"gpu_auto", "gpu_merge", "not_a_gpu_algorithm"}
    runs = d2["algos"]["gpu_auto"]
    assert [r["x"] for r in runs] == [8, 10, 12] and all(r["times"] == [123, 123] for r in runs)
    assert runs[0]["l1d"] == {"rd_access": None, "rd_miss": None, "wr_access": None, "wr_miss": None}
    assert d2["algos"]["not_a_gpu_algorithm"] == []
    assert any("unknown algorithm not_a_gpu_algorithm" in m for m in logs)
    assert ("gpu_svs", 4) in seen
    json.dumps(res)  # serialisable
    # a chosen experiment only
    res = ex.run(exp, root, experiments=["ek"], timers=fake, log=lambda m: None)
    assert set(res["datasets"]) == {"dk"}


@pytest.mark.gpu
def test_registered_timers_run(small, ctx):
    exp, root = small
    ex.generate(exp, root)
    exp["algorithm_sets"]["two"] = list(ex.TIMER_NAMES[:5]) + ["gpu_bsr"]
    for e in exp["experiment"]:
        if e.get("algorithms") == ["gpu_svs"]:
            e["algorithms"] = ["gpu_svs", "gpu_small_adaptive"]
    res = ex.run(exp, root, ctx=ctx, warmup_s=0.0, log=lambda m: None)
    assert res["datasets"]["dk"]["algos"]["gpu_small_adaptive"], "k-set timer did not run"
    for d in res["datasets"].values():
        for name, runs in d["algos"].items():
            assert runs and all(t > 0 for r in runs for t in r["times"]), name
    res = ex.run(exp, root, ctx=ctx, count_only=True, warmup_s=0.0, log=lambda m: None)
    assert res["datasets"]["dk"]["algos"]["gpu_svs"][0]["times"][0] > 0
