"""Hotness-block model sync between replicas (dsgl.hpp:548-781): the row draw, the exchange
over a process group (two gloo ranks on CPU), and the device gather / scatter."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

import sgns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
M64 = (1 << 64) - 1
G = 0x9E3779B97F4A7C15


def mix64(z):
    z = (z + G) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def python_sync_rows(cn_sorted, seed, rnd):
    """One row per block of equal counts, every block but the last (dsgl.hpp:493-509,
    645-711), drawn from the (seed, round) stream."""
    starts = [0] + [r for r in range(1, len(cn_sorted)) if cn_sorted[r] != cn_sorted[r - 1]]
    base = mix64(seed ^ ((rnd * G) & M64))
    rows = []
    for j in range(1, len(starts)):
        r = mix64((base + j * G) & M64)
        rows.append(starts[j - 1] + (((r >> 32) * (starts[j] - starts[j - 1])) >> 32))
    return rows


def test_sync_rows_follow_the_block_rule(sgns_lib):
    rng = np.random.default_rng(3)
    cn = np.sort(rng.zipf(1.8, 5000).astype(np.int32))[::-1].copy()
    for seed, rnd in ((1, 0), (7, 3), (2 ** 63 + 5, 11)):
        rows = sgns.internal_sync_rows(cn, seed, rnd)
        assert rows.tolist() == python_sync_rows(cn.tolist(), seed, rnd)
        # one row per block, inside it, blocks in order, the last block never drawn
        assert len(rows) == len(np.unique(cn)) - 1
        assert all(cn[r] == c for r, c in zip(rows, np.unique(cn)[::-1][:-1]))
    assert sgns.internal_sync_rows(cn, 1, 0, full=True).tolist() == list(range(5000))
    assert sgns.internal_sync_rows(np.full(10, 4, np.int32), 1, 0).tolist() == []  # one block: nothing


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _exchange(rank, ws, port, V, d):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "gdistger-re_gb300")]
    import torch
    import torch.distributed as dist
    import sgns as lib

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    tables = [torch.tensor(np.random.default_rng(100 * rank + w).standard_normal((V, d)), dtype=torch.float32)
              for w in (0, 1)]
    before = [t.clone() for t in tables]
    cn = np.repeat(np.arange(40, 0, -1), 5).astype(np.int32)  # 40 blocks of 5 rows
    rows = torch.from_numpy(lib.internal_sync_rows(cn, 9, 2)).long()

    def gather(which, r):
        return tables[which][r].clone()

    def scatter(which, r, buf, world):
        tables[which][r] = buf / world

    lib.hot_row_sync(rows, gather, scatter, ws, lambda b: dist.all_reduce(b, op=dist.ReduceOp.SUM))
    # every replica now holds the average of the replicas' rows (fp32 sum / count), the rest
    # of each table is untouched
    allb = [[torch.empty_like(t) for _ in range(ws)] for t in before]
    for w in (0, 1):
        dist.all_gather(allb[w], before[w])
        mean = sum(allb[w][k][rows] for k in range(ws)) / ws
        assert torch.equal(tables[w][rows], mean)
        mask = torch.ones(V, dtype=torch.bool)
        mask[rows] = False
        assert torch.equal(tables[w][mask], before[w][mask])
    got = [torch.empty_like(tables[0]) for _ in range(ws)]
    dist.all_gather(got, tables[0])
    assert all(torch.equal(got[0][rows], g[rows]) for g in got)
    dist.barrier()
    dist.destroy_process_group()


def test_exchange_averages_rows_over_two_gloo_ranks(sgns_lib):
    mp.spawn(_exchange, args=(2, _free_port(), 200, 16), nprocs=2, join=True)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["fp32", "bf16"])
def test_gpu_gather_scatter_and_rows(storage, sgns_lib):
    import torch

    V, d = 3000, 64
    rng = np.random.default_rng(5)
    counts = rng.zipf(1.7, V).astype(np.int32)
    with sgns.Trainer(size=d, storage=storage, table_size=100000, debug=0) as t:
        t.set_vocab(counts)
        wih = t.embeddings(0)
        rows = t.sync_rows(4, 1)
        cn_sorted = counts[t.order()]
        assert rows.tolist() == sgns.internal_sync_rows(cn_sorted, 4, 1).tolist()
        r = torch.from_numpy(rows).cuda()
        buf = torch.empty((len(rows), d), device="cuda")
        t.gather_rows(0, r, buf)
        assert np.array_equal(buf.cpu().numpy(), wih[rows])
        new = rng.standard_normal((len(rows), d)).astype(np.float32)
        t.scatter_rows(0, r, torch.from_numpy(new).cuda(), 3.0)
        after = t.embeddings(0)
        want = new / np.float32(3.0)
        if storage == "bf16":  # round to nearest even
            u = want.view(np.uint32).astype(np.uint64)
            want = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16).view(np.float32)
        assert np.array_equal(after[rows], want)
        mask = np.ones(V, bool)
        mask[rows] = False
        assert np.array_equal(after[mask], wih[mask])
