"""The multi-GPU path of bench.py on the CPU: two `gloo` ranks.

Particles are independent and the reference seeds particle i with
seed + i, so rank r's shard [first, first + n) is a run with seed + first.
Each rank runs the oracle on its shard (the last shard takes the remainder);
the shards, gathered, must equal one run of all particles bit for bit.  The
bench's max-over-ranks timing reduction and barrier run on the same group.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
N_TOTAL, TF = 11, 0.01


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path[:0] = [str(REPO), str(REPO / "tests")]
    import torch.distributed as dist
    import bench
    from _oracle import Oracle, Options
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    first, n = bench.shard(N_TOTAL, w, r)
    opt = bench.workload_options(n, TF, first)
    _, out = Oracle().run_sample(Options.from_buffer_copy(bytes(opt)), 0, n, threads=1)
    gathered = [None] * w
    dist.all_gather_object(gathered, (first, n, {k: out[k] for k in ("S", "pos", "n_bounce", "n_steps")}))
    peak = bench.max_over_ranks(w, float(r + 1))
    bench.barrier(w)
    if r == 0:
        np.save(Path(out_dir) / "gathered.npy", np.array([gathered, peak], dtype=object), allow_pickle=True)
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_single_rank_run(oracle, tmp_path):
    pytest.importorskip("torch")
    import socket
    import torch.multiprocessing as mp
    sys.path.insert(0, str(REPO))
    import bench
    from _oracle import Options
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    gathered, peak = np.load(tmp_path / "gathered.npy", allow_pickle=True)
    assert peak == 2.0
    assert [(f, n) for f, n, _ in gathered] == [(0, 5), (5, 6)]
    _, full = oracle.run_sample(Options.from_buffer_copy(bytes(bench.workload_options(N_TOTAL, TF, 0))), 0, N_TOTAL,
                                threads=1)
    for k in ("S", "pos", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(np.concatenate([g[k] for _, _, g in gathered]), full[k], err_msg=k)
