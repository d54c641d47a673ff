"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

On N GPUs every rank runs its own shard of channels (independent integrations,
no data-path collective); the job's time is the slowest rank's, reduced with
an all-reduce MAX, and the value counts every rank's channels (weak scaling).
"""
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, "cpu")
        per_step, value = bench.whole_job_value(ms, world, 5, bench.C)
        q.put((rank, ms, per_step, value))
    finally:
        dist.destroy_process_group()


def test_two_rank_timing_is_slowest_rank_and_value_counts_all_shards():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sys.path.insert(0, str(REPO))
    import bench
    for rank, ms, per_step, value in results:
        assert ms == 20.0  # rank 1's 20 ms, on both ranks
        assert per_step == 4.0
        assert np.isclose(value, 2 * bench.C / 4e-3)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(REPO))
    import bench
    assert bench.max_over_ranks(7.5, 1, "cpu") == 7.5
    assert bench.whole_job_value(30.0, 1, 10, 384) == (3.0, 384 / 3e-3)


def test_shards_are_independent_integrations():
    """Each rank seeds its own integration (make_inputs(seed=rank))."""
    sys.path.insert(0, str(REPO))
    import bench
    import sf_oracle as orc
    sh = orc.Shape(4, bench.F, bench.TP, bench.R, bench.RPP, 2, bench.B)
    a, _, _ = orc.synth_inputs(sh, seed=0)
    b, _, _ = orc.synth_inputs(sh, seed=1)
    assert not np.array_equal(a, b)


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, timeout=120, env=env)
    assert res.returncode == 0
    assert res.stdout.strip() == ""
