"""bench.py's CPU baseline leg on the host: the reference's own CPU kernel (or the oracle restatement where it
cannot be built) on sampled replicas of the benchmarked ensemble, at all host threads and at the reference's
default thread count (4 x cores, include/readdy/common/common.h:80-95), with the keys the bench line reports."""
import os

import bench


def test_cpu_baseline_reports_both_thread_counts():
    ns, boxes, pos, types = bench.ensemble(2024, 32)
    v, n_run, d = bench.reference_cpu(ns, boxes, pos, types, 2024, steps=3, warmup=1, budget_s=10.0)
    cores = os.cpu_count() or 1
    assert v > 0 and n_run > 0
    assert d["value"] == v and d["unit"] == bench.UNIT and d["cores"] == cores and d["threads"] == cores
    assert d["kind"] in ("reference", "port")
    assert d["reference_default_threads"] == 4 * cores
    if d["kind"] == "reference":
        assert d["value_at_default_threads"] > 0
    assert "particle-steps" in d["sample"]
