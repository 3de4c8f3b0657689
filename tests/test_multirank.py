"""Multi-rank plumbing of bench.py on CPU (gloo, world size 2): the barrier and the reductions the
benchmark uses for its max-over-ranks timing, and the dof-balanced split of the batched workload,
which shards its independent systems over ranks with no exchange."""
import json
import os
import socket
import subprocess
import sys

import pytest

from fem_gb300 import problems
from tests.conftest import ROOT


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_batch_shard_partitions_the_plan(world):
    plan = problems.batch_plan(96, seed=0)
    shards = [problems.batch_shard(plan, r, world) for r in range(world)]
    flat = [p for sh in shards for p in sh]
    assert sorted(flat) == sorted(plan) and len(flat) == len(plan)
    for sh in shards:  # plan order kept within a rank
        assert sh == [p for p in plan if p in sh]
    loads = [sum(d for _, d, _ in sh) for sh in shards]
    assert max(loads) - min(loads) <= max(d for _, d, _ in plan)
    assert problems.batch_shard(plan, 0, 1) == plan


WORKER = r"""
import json, os, sys
sys.path.insert(0, os.environ["LINA_ROOT"])
import bench
from fem_gb300 import problems
rank, world, local = bench.dist_info()
bench.init_dist(world)
bench.barrier(world)
out = {"rank": rank, "world": world,
       "sum": bench.sum_over_ranks(rank + 1, world),
       "max": bench.max_over_ranks(10.0 * rank, world),
       "shard": [list(p) for p in problems.batch_shard(problems.batch_plan(12, seed=0), rank, world)]}
bench.barrier(world)
with open(os.path.join(os.environ["LINA_OUT"], "rank%d.json" % rank), "w") as f:
    json.dump(out, f)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    assert torch.distributed.is_gloo_available()
    script = tmp_path / "worker.py"
    script.write_text(WORKER)
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), LINA_ROOT=ROOT, LINA_OUT=str(tmp_path))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    for p in procs:
        out, _ = p.communicate(timeout=600)
        assert p.returncode == 0, out[-3000:]
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    plan = [list(p) for p in problems.batch_plan(12, seed=0)]
    for r in res:
        assert r["world"] == 2 and r["sum"] == 3.0 and r["max"] == 10.0
    assert sorted(res[0]["shard"] + res[1]["shard"]) == sorted(plan)
    assert not any(p in res[1]["shard"] for p in res[0]["shard"])
