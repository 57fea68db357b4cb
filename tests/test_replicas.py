"""The N > 1 host path of bench.py (replicas, no data exchange) on CPU ranks.

Two processes join a gloo group on 127.0.0.1, as torchrun would start them,
and run the reductions bench.py applies to a replica run: the job time is the
slowest rank's, the work the sum of the ranks'.  The pipeline itself runs per
rank on its own pairs, so the oracle stands in for it here (no GPU).
"""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), RTS_DIST_BACKEND="gloo")
    import bench
    import oracle

    bench.dist_init(world)
    # each rank its own small pair (seeded by rank), timed on the host
    import time

    import rtstereo_gb300 as R
    L, Rr, _ = R.synth_pair(0xC3000 + 1000 * rank, 48, 24, 8, 3, 0, 2.0, 4)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    bench.ranks_barrier(world)
    t0 = time.perf_counter()
    dl, dr, mk, _ = oracle.pipeline(oracle.params(D=8), L, Rr, Lc, Rc)
    ms = (time.perf_counter() - t0) * 1e3 + 10.0 * rank  # rank 1 is the slow one
    job_ms = bench.ranks_max([ms], world)[0]
    work = bench.ranks_sum([48 * 24 * 8], world)[0]
    checks = bench.ranks_sum([float(dl.sum()), float(mk.sum())], world)
    bench.ranks_barrier(world)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.array([ms, job_ms, work] + checks))
    bench.ranks_done(world)


@pytest.mark.timeout(300)
def test_two_replica_ranks_reduce_like_the_bench(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn", join=True)
    r = [np.load(tmp_path / f"rank{i}.npy") for i in range(world)]
    # every rank sees the same job figures: the slowest rank's time, the summed work
    assert r[0][1] == r[1][1] == max(r[0][0], r[1][0])
    assert r[0][2] == r[1][2] == world * 48 * 24 * 8
    assert np.array_equal(r[0][3:], r[1][3:])
