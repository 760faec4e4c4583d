"""One gloo rank of tests/test_bench_ranks.py: runs bench.py's multi-rank
host logic on CPU (RANK, WORLD_SIZE, MASTER_ADDR and MASTER_PORT come from
the environment, as torchrun sets them) and prints one JSON line."""
import importlib.util
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _module(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    import torch
    import torch.distributed as dist

    bench = _module("bench", os.path.join(ROOT, "bench.py"))
    scenes = _module("scenes", os.path.join(ROOT, "sparse-voxel-octrees_gb300", "scenes.py"))
    rank, world, local = bench.dist_setup(None)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # each rank traced a different number of rays, in a different time
    units, secs = bench.reduce_over_ranks(torch, 1000 + 7 * rank, 0.5 + rank, "cpu")
    cams = bench.rank_cameras(scenes, 3, rank, (0.5, 0.5, 0.5))
    dist.barrier()
    dist.destroy_process_group()
    print(json.dumps({"rank": rank, "world": world, "local": local, "units": units, "secs": secs,
                      "cams": np.asarray(cams, dtype=np.float64).tolist()}))


if __name__ == "__main__":
    sys.exit(main())
