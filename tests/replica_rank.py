"""One rank of the replica test (tests/test_replicas_gloo.py): run as a process with RANK,
WORLD_SIZE, MASTER_ADDR and MASTER_PORT set; prints one JSON line with its share."""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def unit_checksum(fs, refcpu, u):
    raw, truth = fs.synth.make_dataset(n=64, seed=900 + u)
    sp = fs.synth.sim_param_for(truth, 64)
    return float(np.sum(refcpu.recon_raw(sp, raw, fade=2), dtype=np.float64))


def main():
    import torch.distributed as dist

    import __graft_entry__ as g
    from oracle import refcpu

    fs = g.load_package()
    refcpu.set_threads(1)
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    n_units = int(sys.argv[1])
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = fs.replicas.shard(n_units, rank, world)
    sums = {u: unit_checksum(fs, refcpu, u) for u in mine}
    elapsed = fs.replicas.max_over_ranks(1.0 + rank)
    total = fs.replicas.sum_over_ranks(len(mine))
    dist.destroy_process_group()
    print(json.dumps({"rank": rank, "mine": mine, "sums": sums, "elapsed": elapsed, "total": total}))


if __name__ == "__main__":
    main()
