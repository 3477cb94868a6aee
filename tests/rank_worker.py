"""One rank of the two-rank CPU check of bench.py's multi-rank path (gloo).

Launched by tests/test_multirank_host.py through torch.distributed.run; reads
RANK / WORLD_SIZE / MASTER_* from the environment like bench.py does.
"""

import argparse
import contextlib
import io
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import bench  # noqa: E402
from traffic_assignment_gb300 import synth  # noqa: E402


def main():
    rank, world, _ = bench._env_rank()
    assert world == 2
    dist = bench.Dist(world)
    dist.barrier()
    # max over ranks and the whole-job rate: units of all ranks / slowest time
    assert dist.max(1.0 + rank) == 2.0
    assert dist.sum(10 * (rank + 1)) == 30.0
    rate = bench.whole_job_rate(dist, 100, 2.0 if rank == 0 else 4.0)
    assert rate == 200 / 4.0, rate
    # scenario shards: each rank its own, no data exchange needed to build them
    net, _ = synth.make_small24()
    mine = bench.shard_scenarios(net, 8, rank)
    other = bench.shard_scenarios(net, 8, 1 - rank)
    assert [list(s.links) for s in mine] != [list(s.links) for s in other]
    sig = torch.tensor([float(sum(int(np.sum(s.links)) for s in mine))], dtype=torch.float64)
    got = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.td.all_gather(got, sig)
    assert got[rank].item() == sig.item() and got[0].item() != got[1].item()
    # the reference arm: rank 0 alone runs and prints; the others exit 0 silently
    if rank != 0:
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            rc = bench.run_reference(argparse.Namespace(gpus=2, steps=1, warmup=3), rank, world)
        assert rc == 0 and buf.getvalue() == ""
    dist.barrier()
    dist.close()
    print(f"rank {rank} ok", flush=True)


if __name__ == "__main__":
    main()
