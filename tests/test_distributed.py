"""The N > 1 path of bench.py on CPU: two gloo ranks each take their own seeded ensemble of replicas
(no data exchange) and reduce only the timed region's time (max) and particle-steps (sum)."""
import json
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r, w = bench.init_dist()
    ns, _, pos, _ = bench.ensemble(bench.rank_seed(2024, r), 6)
    bench.barrier(w)
    total = bench.allreduce_sum(float(ns.sum()), w)
    slowest = bench.allreduce_max(1.5 + r, w)
    first = float(pos[0][0, 0])
    with open(os.path.join(out, f"rank{r}.json"), "w") as f:
        json.dump(dict(total=total, slowest=slowest, local=int(ns.sum()), first=first), f)
    bench._dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_particle_steps(tmp_path):
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert res[0]["total"] == res[1]["total"] == res[0]["local"] + res[1]["local"]
    assert res[0]["slowest"] == res[1]["slowest"] == 2.5
    assert res[0]["first"] != res[1]["first"]  # disjoint, independently seeded ensembles
