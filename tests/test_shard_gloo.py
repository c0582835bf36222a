"""The multi-process path of a sharded run, on CPU with the gloo backend (world size 2): each
rank sums the exact fixed-point contributions of its own contiguous range of paths, the ranks
reduce their int64 words with all_reduce, and the finished results equal those of one process
summing every path, bit for bit.  The contributions are synthetic (a hash of the path index),
and each rank splits its words between the hi and lo parts differently, as different block
groupings on different GPUs would."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N_PATH, N_RISK, N_PAY = 1000, 7, 2
N_WORDS = 2 * (N_RISK + 2 * N_PAY + 2)


def contributions(first, count):
    """Exact per-path contributions in units of 2^-60 (Python ints), one per accumulator."""
    out = np.zeros((count, N_WORDS // 2), dtype=object)
    for i in range(count):
        h = (first + i + 1) * 0x9E3779B97F4A7C15 & ((1 << 64) - 1)
        for j in range(N_WORDS // 2):
            h = (h ^ (h >> 29)) * 0xBF58476D1CE4E5B9 & ((1 << 64) - 1)
            out[i, j] = (h % (1 << 44)) - (1 << 43)  # |value| < 2^-16
    return out


def accumulate(contrib, carry_every):
    """hi/lo words of the sums (hi: units of 2^-20), the lo part normalised into hi every
    `carry_every` paths: the same exact total, a different split of the words."""
    acc = np.zeros(N_WORDS, dtype=np.int64)
    for i, row in enumerate(contrib):
        for j, v in enumerate(row):
            acc[2 * j + 1] += int(v)
        if (i + 1) % carry_every == 0:
            c = acc[1::2] >> 40
            acc[0::2] += c
            acc[1::2] -= c << 40
    return acc


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from compfinance_gb300.shard import combine, shard_range
    from compfinance_gb300.api import results_from_raw
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    first, count = shard_range(N_PATH, rank, world)
    acc = accumulate(contributions(first, count), carry_every=3 + 4 * rank)
    total = combine(acc)
    v, e, agg, r = results_from_raw(total, N_RISK, N_PAY, N_PATH)
    q.put((rank, first, count, v.tolist(), e.tolist(), agg, r.tolist()))
    dist.destroy_process_group()


def test_sharded_reduction_is_exact():
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    from compfinance_gb300.api import results_from_raw
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # shards are contiguous, 64-aligned and cover the run
    assert got[0][1] == 0 and got[0][2] + got[1][2] == N_PATH and got[1][1] == got[0][2] and got[1][1] % 64 == 0
    # one process over every path, a third split of the words
    full = accumulate(contributions(0, N_PATH), carry_every=1)
    v, e, agg, r = results_from_raw(full, N_RISK, N_PAY, N_PATH)
    for rank in range(2):
        assert got[rank][3] == v.tolist() and got[rank][4] == e.tolist()
        assert got[rank][5] == agg and got[rank][6] == r.tolist()
