"""Co-optimal path counts on the device against the oracle's enumeration (needs a GPU).

pa_result_path_counts counts, per lane of an all-optimal solve, the results the reference's
depth-first enumeration (solver.h:1647-1716) yields when duplicates are kept (return_dup).
Here the count of every pair is compared with the number of alignments the oracle's
iterator yields with return_dup=True, and with the GPU iterator's own enumeration, on
tie-rich cases: small alphabets, integer scores, every locality, linear and affine gaps,
both directions, the group widths of the group mode and the stripe-chained mode, empty
pairs, and pairs whose local optimum is 0 (no seed: count 0).
"""

import zlib

import numpy as np
import pytest

from _cases import Gap, options, pack, random_pairs

pytestmark = pytest.mark.gpu

CAP = 20000  # enumerations longer than this are not compared (counted only)


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


def _count(it):
    n = 0
    while n <= CAP and it.next() is not None:
        n += 1
    return n


def _pairs(rng, n):
    pairs = random_pairs(rng, n, 1, 26, alphabet=2, related=0.5)
    pairs[0] = (pairs[0][0][:0], pairs[0][1])
    pairs[1] = (pairs[1][0], pairs[1][1][:0])
    pairs[2] = (np.zeros(5, np.uint32), np.ones(7, np.uint32))    # no match at all
    pairs[3] = (np.zeros(20, np.uint32), np.zeros(23, np.uint32))  # one letter: many gap placements
    return pairs


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("gap", ["linear", "affine"])
@pytest.mark.parametrize("direction", ["maximize", "minimize"])
@pytest.mark.parametrize("mode", ["G8", "G32", "chained"])
def test_path_counts_equal_enumeration(monkeypatch, gpu_alg, oracle_alg, locality, gap, direction, mode):
    if mode == "chained":
        monkeypatch.setenv("PA_DP_MODE", "units")
    else:
        monkeypatch.setenv("PA_GROUP_WIDTH", mode[1:])
    rng = np.random.default_rng(zlib.crc32(f"count/{locality}/{gap}/{direction}/{mode}".encode()))
    pairs = _pairs(rng, 40)
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    if direction == "minimize":
        table = -table
    g = Gap("linear", 1.0) if gap == "linear" else Gap("affine", 2.0, 1.0)
    o = dict(options(gpu_alg, locality=locality, direction=direction, count="all", gap=g, return_dup=True),
             batch_size=n, batch=True)
    cap = (a.shape[1], b.shape[1])
    gs = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o))
    its = gs.solve_indexed_for_alignment_iterator(a, b, table, ln)
    counts = [it.path_count() for it in its]
    os_ = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o))
    oits = os_.solve_indexed_for_alignment_iterator(a, b, table, ln)
    compared = 0
    for k in range(n):
        want = _count(oits[k])
        if want > CAP:
            assert counts[k] > CAP, (k, counts[k])
            continue
        assert counts[k] == want, (k, counts[k], want, ln[:, k])
        assert _count(its[k]) == want, k
        compared += 1
    assert compared >= n // 2
    if locality == "local":
        assert counts[2] == 0  # optimum 0: no seed


@pytest.mark.parametrize("count_mode", ["chain", "group"])
def test_path_counts_of_multi_stripe_pairs(monkeypatch, gpu_alg, oracle_alg, count_mode):
    """Pairs of 513-800 rows (three or four 256-row stripes of the stripe-chained layout): the
    count with a warp per stripe, stripes chained (and, for comparison, a group per pair)
    equals the oracle's enumeration.  A continuous score table keeps ties -- and so the
    enumerations -- small."""
    monkeypatch.setenv("PA_DP_MODE", "units")
    monkeypatch.setenv("PA_COUNT_MODE", count_mode)
    rng = np.random.default_rng(6161)
    n = 12
    pairs = [(rng.integers(0, 3, size=int(rng.integers(513, 801))).astype(np.uint32),
              rng.integers(0, 3, size=int(rng.integers(20, 61))).astype(np.uint32)) for _ in range(n)]
    pairs[0] = (pairs[0][0], pairs[0][1][:0])   # empty t
    a, b, ln = pack(pairs, n)
    table = np.round(rng.normal(size=(3, 3)), 1).astype(np.float32)
    for locality, gap in (("global", Gap("affine", 2.0, 0.5)), ("local", Gap("affine", 2.0, 0.5)),
                          ("semiglobal", Gap("linear", 1.0))):
        o = dict(options(gpu_alg, locality=locality, count="all", gap=gap, return_dup=True), batch_size=n, batch=True)
        cap = (a.shape[1], b.shape[1])
        gs = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o))
        its = gs.solve_indexed_for_alignment_iterator(a, b, table, ln)
        assert gs.last_plan()["kernel"] == "stripe-chained", gs.last_plan()
        counts = [it.path_count() for it in its]
        os_ = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o))
        oits = os_.solve_indexed_for_alignment_iterator(a, b, table, ln)
        for k in range(n):
            want = _count(oits[k])
            if want > CAP:
                assert counts[k] > CAP, (locality, k, counts[k])
            else:
                assert counts[k] == want, (locality, k, counts[k], want)
