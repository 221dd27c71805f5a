"""bench.py under torchrun, without a GPU: two gloo ranks on this host. Instances shard by rank
with no exchange (each rank's shard is exactly its slice of the whole batch), the timed region's
times and counts reduce across ranks (max / sum), and only rank 0 prints its JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

CHILD = r'''
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
from sayram2d_gb300 import cases
R = bench.Ranks()
out = {"rank": R.rank, "world": R.world}
out["max"] = R.max(1.5 + R.rank)
out["sum"] = R.sum(10 * (R.rank + 1))
out["min"] = -R.max(-(3.0 - R.rank))
shard = cases.batch_shard(3, 7, 1e-2, R.rank, R.world)
whole = cases.batch_problems(3 * R.world, 7, 1e-2)[3 * R.rank:3 * (R.rank + 1)]
out["shard_equal"] = all(a.nx == b.nx and a.ny == b.ny and (a.G == b.G).all() and (a.Dxy == b.Dxy).all()
                         and (a.f0 == b.f0).all() for a, b in zip(shard, whole))
out["shard_sizes"] = [(p.nx, p.ny) for p in shard]
R.barrier()
with open(os.path.join(sys.argv[2], f"rank{R.rank}.json"), "w") as fh:
    json.dump(out, fh)
R.emit({"printed_by": R.rank})
R.close()
'''


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT, str(tmp_path)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=240) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
    r = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(2)]
    for k in range(2):
        assert r[k]["world"] == 2 and r[k]["rank"] == k
        assert r[k]["max"] == 2.5 and r[k]["sum"] == 30.0 and r[k]["min"] == 2.0
        assert r[k]["shard_equal"]
    assert r[0]["shard_sizes"] != r[1]["shard_sizes"]  # disjoint slices of the seeded batch
    # only rank 0 prints its line
    assert json.loads(outs[0][0].strip().splitlines()[-1]) == {"printed_by": 0}
    assert outs[1][0].strip() == ""


def test_gpus_must_match_the_launch(monkeypatch):
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py", "--gpus", "2"])
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    with pytest.raises(SystemExit, match="torchrun"):
        bench.main()


def test_single_process_needs_no_process_group(monkeypatch):
    import bench

    monkeypatch.delenv("WORLD_SIZE", raising=False)
    R = bench.Ranks()
    assert R.world == 1 and R.dist is None
    assert R.max(3.0) == 3.0 and R.sum(2.0) == 2.0
    R.close()
