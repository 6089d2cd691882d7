"""The multi-rank path on CPU: two gloo ranks shard a batch by object, gather the
per-object results in order and reduce the step time (no GPU involved)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from gpu_lomb_scargle_gb300 import shard, synth


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, offsets, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        o0, o1, r0, r1, local = shard.local_batch(offsets, rank, world)
        # stand-in per-object results: what the GPU would return for these objects
        idx = np.arange(o0, o1) * 7 % 1000
        pw = np.arange(o0, o1) / 10.0
        gi, gp = shard.gather_best(idx, pw, o0, len(offsets) - 1)
        t = shard.max_over_ranks(1.0 + rank)
        q.put((rank, o0, o1, r0, r1, int(local[-1]), gi.tolist(), gp.tolist(), t))
    finally:
        dist.destroy_process_group()


def test_shard_ranges_cover_all_objects_balanced():
    w = synth.lognormal_batch(seed=1, n_obj=999, n_freq=10)
    ranges = [shard.shard_range(w.offsets, r, 4) for r in range(4)]
    assert ranges[0][0] == 0 and ranges[-1][1] == 999
    assert all(ranges[i][1] == ranges[i + 1][0] for i in range(3))
    rows = [int(w.offsets[b] - w.offsets[a]) for a, b in ranges]
    assert max(rows) - min(rows) < 2 * 1500  # within two of the largest objects


@pytest.mark.parametrize("world", [2])
def test_two_gloo_ranks_gather_and_max_time(world):
    w = synth.lognormal_batch(seed=2, n_obj=57, n_freq=10)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, w.offsets, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert out[0][1] == 0 and out[-1][2] == 57 and out[0][2] == out[1][1]
    for rank, o0, o1, r0, r1, nrows, gi, gp, t in out:
        assert nrows == r1 - r0 == int(w.offsets[o1] - w.offsets[o0])
        assert gi == (np.arange(57) * 7 % 1000).tolist()  # every rank sees all objects in order
        assert np.allclose(gp, np.arange(57) / 10.0)
        assert t == float(world)  # max over ranks of 1 + rank
