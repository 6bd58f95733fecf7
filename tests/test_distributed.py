"""Multi-rank host logic with two gloo ranks on the CPU: disjoint event
ranges that cover the batch, and the merge of averaged profiles equal to a
one-process mean (the only reduction of the data path)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from supermc_gb300.distributed import event_range, step_events


def test_event_ranges_partition_the_batch():
    for total in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            ids = []
            for r in range(world):
                f, n = event_range(100, total, r, world)
                ids += list(range(f, f + n))
            assert ids == list(range(100, 100 + total))
    seen = {step_events(s, r, 4, 10) for s in range(3) for r in range(4)}
    assert len(seen) == 12 and all(v % 10 == 0 for v in seen)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from supermc_gb300.distributed import max_over_ranks, merge_means
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(rank)
    # per-rank binned means of a few "events" (3 bins of 4 x 5 cells) and an unbinned mean
    counts = np.array([2 + rank, 0, 5 - rank])
    grids = [rng.random((c, 4, 5)) for c in counts]
    means = np.stack([g.mean(axis=0) if len(g) else np.zeros((4, 5)) for g in grids])
    merged, tot = merge_means(means, counts)
    flat = np.concatenate(grids)
    m2, t2 = merge_means(flat.mean(axis=0), len(flat))
    slow = max_over_ranks(1.5 + rank)
    q.put((rank, grids, merged, tot, m2, t2, slow))
    dist.destroy_process_group()


def test_merge_of_averaged_profiles_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in procs], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    all_grids = [np.concatenate([res[0][1][b], res[1][1][b]]) for b in range(3)]
    want = np.stack([g.mean(axis=0) if len(g) else np.zeros((4, 5)) for g in all_grids])
    for _, _, merged, tot, m2, t2, slow in res:
        np.testing.assert_allclose(merged, want, rtol=1e-12, atol=1e-15)
        np.testing.assert_array_equal(tot, [len(g) for g in all_grids])
        flat = np.concatenate([np.concatenate(r[1]) for r in res])
        np.testing.assert_allclose(m2, flat.mean(axis=0), rtol=1e-12)
        assert t2 == len(flat)
        assert slow == 2.5
