"""The N > 1 host path of bench.py on CPU: each rank is one independent replica (the iteration map
is not sharded across GPUs in this build); the ranks meet at a barrier around the timed region and
rank 0 reports the maximum time over ranks.  Two gloo ranks on 127.0.0.1, no GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, loc = bench.dist_env()
    assert (r, w, loc) == (rank, world, rank)
    d = bench.Dist(w)
    d.barrier()
    m = d.max(float(rank) + 0.5)  # each rank's own "time"; the report takes the maximum
    d.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(m))
    d.dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_max(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(2)]
    assert vals == [1.5, 1.5]
