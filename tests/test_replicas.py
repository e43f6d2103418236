"""`bench.py --gpus N` runs N independent replicas ("replicas only": the path does
not shard across GPUs here). The host side of that path -- one process per rank
over gloo, a barrier around the timed region, the slowest rank's time -- is
checked on the CPU with two ranks."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

WORKER = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
d = bench.Dist()
d.barrier()
t = d.max(0.5 * (d.rank + 1))
d.barrier()
print(json.dumps({"world": d.world, "rank": d.rank, "max": t}))
d.close()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_agree_on_the_slowest_time():
    pytest.importorskip("torch")
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER, str(ROOT)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    out = []
    for p in procs:
        stdout, stderr = p.communicate(timeout=120)
        assert p.returncode == 0, stderr[-2000:]
        out.append(json.loads(stdout.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in out) == [0, 1]
    assert all(o["world"] == 2 and o["max"] == 1.0 for o in out), out


def test_one_rank_needs_no_process_group():
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "-c", WORKER, str(ROOT)], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    o = json.loads(r.stdout.strip().splitlines()[-1])
    assert o == {"world": 1, "rank": 0, "max": 0.5}
