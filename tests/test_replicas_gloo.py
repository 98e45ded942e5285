"""Multi-GPU form = independent replicas: each rank takes a disjoint share of the datasets
and the only cross-rank step is the max of the elapsed times (and the sum of the units)
for reporting. Checked here with world_size 2 over gloo on the CPU, each rank
reconstructing its share with the oracle at a small size: the shares cover every dataset
exactly once and the gathered checksums equal a single-process run."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_shard_is_a_balanced_partition(fs):
    for n in (0, 1, 7, 64):
        for w in (1, 2, 3, 8):
            parts = [fs.replicas.shard(n, r, w) for r in range(w)]
            flat = [u for p in parts for u in p]
            assert flat == list(range(n))
            assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        fs.replicas.shard(4, 2, 2)


def test_two_rank_replicas_over_gloo(fs):
    import json
    import subprocess
    import sys

    from oracle import refcpu

    from replica_rank import unit_checksum

    refcpu.build()
    port = _free_port()
    n_units = 5
    here = os.path.dirname(os.path.abspath(__file__))
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.join(here, "replica_rank.py"), str(n_units)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    res = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        res.append(json.loads(out.strip().splitlines()[-1]))
    res.sort(key=lambda r: r["rank"])
    assert [u for r in res for u in r["mine"]] == list(range(n_units))
    assert all(r["elapsed"] == 2.0 for r in res)  # max over ranks
    assert all(r["total"] == n_units for r in res)  # units processed by all ranks
    refcpu.set_threads(1)
    for r in res:
        for u in r["mine"]:
            assert r["sums"][str(u)] == unit_checksum(fs, refcpu, u)
