"""One bag over several ranks (CPU, torch.distributed gloo, world sizes 2 and 3).

shard_pairs splits a bag by cells with no communication and gather_results puts every
rank's scores and maps back in bag order.  Here gloo ranks each solve their share of a
bag of small pairs with the oracle (standing in for each rank's GPU) and the gathered
results must equal the oracle's solve of the whole bag; the split itself must cover every
pair once and balance the cells.
"""

import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from pyalign_gb300.shard import gather_results, shard_pairs


def _bag(seed=5, n=57):
    rng = np.random.default_rng(seed)
    ls = rng.integers(0, 40, n)
    lt = rng.integers(0, 40, n)
    a = rng.integers(0, 4, (n, 40)).astype(np.uint32)
    b = rng.integers(0, 4, (n, 40)).astype(np.uint32)
    table = np.full((4, 4), -1.0, np.float32)
    np.fill_diagonal(table, 2.0)
    return a, b, ls, lt, table


def _oracle_solve(a, b, ls, lt, table):
    """Scores and concatenated maps of the pairs with the oracle (local affine 5/2)."""
    import oracle.algorithm as oalg
    from _cases import Gap, options
    n = len(ls)
    o = dict(options(oalg, locality="local", gap=Gap("affine", 5.0, 2.0)), batch_size=max(n, 1), batch=True)
    solver = oalg.m16.create_solver(40, 40, oalg.m16.create_options(o))
    res = solver.solve_indexed_for_alignment(a, b, table, np.stack([ls, lt]).astype(np.uint16))
    scores = np.array([r.score for r in res], np.float32)
    maps = [np.asarray(r.s_to_t if ls[k] <= lt[k] else r.t_to_s, np.int32) for k, r in enumerate(res)]
    sizes = np.array([len(m) for m in maps], np.int64)
    return scores, (np.concatenate(maps) if maps else np.zeros(0, np.int32)), sizes


def test_split_covers_every_pair_once_and_balances_cells():
    rng = np.random.default_rng(1)
    ls, lt = rng.integers(0, 1000, 5000), rng.integers(0, 1000, 5000)
    for world in (1, 2, 3, 8):
        parts = [shard_pairs(ls, lt, world, r) for r in range(world)]
        allidx = np.concatenate(parts)
        assert np.array_equal(np.sort(allidx), np.arange(5000))
        loads = [int((ls[p] * lt[p]).sum()) for p in parts]
        assert max(loads) - min(loads) <= int((ls * lt).max()), (world, loads)
    with pytest.raises(ValueError):
        shard_pairs(ls, lt, 2, 2)


def _rank(rank, world, port, out, n):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b, ls, lt, table = _bag(n=n)
        idx = shard_pairs(ls, lt, world, rank)
        if len(idx):
            sc, mp_, sizes = _oracle_solve(a[idx], b[idx], ls[idx], lt[idx], table)
        else:
            sc, mp_, sizes = [], [], []   # a rank with no pairs (more ranks than pairs)
        all_sc, all_mp, offs = gather_results(idx, sc, mp_, sizes, len(ls))
        out.put((rank, len(idx), all_sc, all_mp, offs))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,n", [(2, 57), (3, 2)])
def test_gloo_ranks_gather_the_whole_bag(world, n):
    """Two ranks over 57 pairs, and three ranks over 2 pairs (one rank solves nothing and
    passes empty lists): every rank ends with the whole bag's results in bag order."""
    pytest.importorskip("torch")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q, n)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b, ls, lt, table = _bag(n=n)
    want_sc, want_mp, want_sizes = _oracle_solve(a, b, ls, lt, table)
    assert sum(k for _, k, _, _, _ in got) == n
    for rank, _, sc, mp_, offs in got:
        assert sc.dtype == want_sc.dtype and mp_.dtype == want_mp.dtype, rank
        assert np.array_equal(sc, want_sc), rank
        assert np.array_equal(mp_, want_mp), rank
        assert np.array_equal(offs, np.concatenate([[0], np.cumsum(want_sizes)[:-1]])), rank
