"""The multi-process path of bench.py on CPU: two gloo ranks on 127.0.0.1,
each with its own replica set, agree on the slowest rank's step time."""
import os
import re
import subprocess
import sys
import textwrap

import pytest

from dmdgb import sharding, systems

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_round_robin():
    parts = [sharding.shard(10, 3, r) for r in range(3)]
    assert parts == [[0, 3, 6, 9], [1, 4, 7], [2, 5, 8]]
    assert sorted(sum(parts, [])) == list(range(10))
    with pytest.raises(ValueError):
        sharding.shard(4, 2, 2)


def test_rank_workloads_differ():
    a = systems.config_c3(32, seed=sharding.replica_seed(0))
    b = systems.config_c3(32, seed=sharding.replica_seed(1))
    assert [s.n_beads for s in a] != [s.n_beads for s in b]


def test_two_gloo_ranks_max(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import os, sys
        sys.path.insert(0, {repr(os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300"))})
        import torch.distributed as dist
        from dmdgb import sharding
        dist.init_process_group("gloo")
        r = dist.get_rank()
        v = sharding.max_over_ranks(1.5 + r)
        print(f"rank {{r}} max {{v}}", flush=True)
        dist.destroy_process_group()
    """))
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29541", str(script)]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=240, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    found = sorted(re.findall(r"rank (\d) max ([0-9.]+)", out.stdout))
    assert found == [("0", "2.5"), ("1", "2.5")], out.stdout
