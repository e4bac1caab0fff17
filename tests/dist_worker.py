"""Worker for tests/test_dist.py, launched by torch.distributed.run with
world_size 2 on the gloo backend: bench.py's barrier and max-over-ranks
helpers, as its N>1 timing uses them."""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

rank, world, d = bench.dist_setup(2)
bench.barrier(d)
mx = bench.allmax(d, 1.5 + rank)
bench.barrier(d)
print(json.dumps({"rank": rank, "world": world, "max": mx}), flush=True)
if d is not None:
    d.destroy_process_group()
