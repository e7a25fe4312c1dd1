"""The first k optimal alignments of every lane, enumerated on the device (needs a GPU).

pa_result_first_alignments runs the reference's depth-first search over the all-optimal
traceback lists (solver.h:1647-1716) for every lane of a result at once, one warp per lane.
Its results must be the host search's (pa_iterator_next) result for result, in order --
maps, walks, de-duplication and exhaustion -- and the oracle's iterator's maps.  Covered:
tie-rich pairs (two letters, integer scores) of every locality, linear and affine gaps,
both directions, de-duplication on and off, the group and stripe-chained mask layouts,
multi-stripe pairs, empty pairs and local pairs without a positive optimum; the retry
protocol when a lane's search stack or seed list is too small (PA_ENUM_STACK,
PA_ENUM_SEEDS force tiny ones); the Python iterators, which serve the device results
first and then resume the host search after them (PA_ENUM_FIRST sets how many); and the
alignment and solution codomains of all-optimal solvers, whose first results come from the
same enumeration.
"""

import ctypes
import zlib

import numpy as np
import pytest

from _cases import Gap, options, pack, random_pairs

pytestmark = pytest.mark.gpu

K = 40


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


def _pairs(rng, n, lo=1, hi=26):
    pairs = random_pairs(rng, n, lo, hi, alphabet=2, related=0.5)
    pairs[0] = (pairs[0][0][:0], pairs[0][1])
    pairs[1] = (pairs[1][0], pairs[1][1][:0])
    pairs[2] = (np.zeros(5, np.uint32), np.ones(7, np.uint32))    # no match: local optimum 0
    pairs[3] = (np.zeros(20, np.uint32), np.zeros(23, np.uint32))  # one letter: many gap placements
    pairs[4] = (np.tile([0, 1], 9).astype(np.uint32), np.tile([1, 0], 8).astype(np.uint32))  # many local seeds
    return pairs


def _host_search(alg, res, lane, k, ls, lt):
    """The first k results of the host search (pa_iterator_next) of one lane."""
    L = alg.lib()
    h = alg._P()
    alg.check(L.pa_result_iterator(res.ptr, lane, ctypes.byref(h)))
    out = []
    try:
        for _ in range(k):
            sc = ctypes.c_float(0)
            mp = np.zeros(min(ls, lt), np.int32)
            path = np.zeros((ls + lt + 4, 2), np.int32)
            n = ctypes.c_int64(0)
            if not L.pa_iterator_next(h, ctypes.byref(sc), alg._ip(mp), alg._ip(path), ctypes.byref(n)):
                break
            out.append((mp, path[:n.value].copy()))
    finally:
        L.pa_iterator_destroy(h)
    return out


def _solve(alg, pairs, locality, gap, direction, remove_dup, table):
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    o = dict(options(alg, locality=locality, direction=direction, count="all", gap=gap,
                     return_dup=not remove_dup), batch_size=n, batch=True)
    cap = (a.shape[1], b.shape[1])
    solver = alg.m16.create_solver(*cap, alg.m16.create_options(o))
    its = solver.solve_indexed_for_alignment_iterator(a, b, table, ln)
    return solver, its, ln, o, cap, (a, b)


def _compare_with_host(alg, its, ln, k):
    res = its[0]._res
    f = alg.FirstAlignments(res, k, with_paths=True)
    for lane in range(len(its)):
        ls, lt = int(ln[0, lane]), int(ln[1, lane])
        want = _host_search(alg, res, lane, k, ls, lt)
        assert int(f.counts[lane]) == len(want), (lane, int(f.counts[lane]), len(want))
        for j, (mp, path) in enumerate(want):
            gm, gp = f.alignment(lane, j)
            assert np.array_equal(gm, mp), (lane, j)
            assert np.array_equal(gp, path), (lane, j)
    return f


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("gap", ["linear", "affine"])
@pytest.mark.parametrize("direction", ["maximize", "minimize"])
@pytest.mark.parametrize("remove_dup", [True, False])
@pytest.mark.parametrize("mode", ["G8", "chained"])
def test_first_alignments_match_host_search(monkeypatch, gpu_alg, oracle_alg, locality, gap, direction,
                                            remove_dup, mode):
    if mode == "chained":
        monkeypatch.setenv("PA_DP_MODE", "units")
    else:
        monkeypatch.setenv("PA_GROUP_WIDTH", mode[1:])
    rng = np.random.default_rng(zlib.crc32(f"enum/{locality}/{gap}/{direction}/{remove_dup}/{mode}".encode()))
    pairs = _pairs(rng, 36)
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    if direction == "minimize":
        table = -table
    g = Gap("linear", 1.0) if gap == "linear" else Gap("affine", 2.0, 1.0)
    solver, its, ln, o, cap, (a, b) = _solve(gpu_alg, pairs, locality, g, direction, remove_dup, table)
    f = _compare_with_host(gpu_alg, its, ln, K)
    # and the oracle's iterators, map for map
    osol = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o))
    oits = osol.solve_indexed_for_alignment_iterator(a, b, table, ln)
    for lane in range(len(pairs)):
        ls, lt = int(ln[0, lane]), int(ln[1, lane])
        for j in range(int(f.counts[lane])):
            x = oits[lane].next()
            assert x is not None, (lane, j)
            want = x.s_to_t if ls <= lt else x.t_to_s
            assert np.array_equal(f.alignment(lane, j)[0], np.asarray(want)), (lane, j)
        if f.counts[lane] < K:
            assert oits[lane].next() is None, lane
    if locality == "local":
        assert f.counts[2] == 0  # optimum 0: no seed


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_first_alignments_of_multi_stripe_pairs(monkeypatch, gpu_alg, locality):
    """Pairs of 513-800 rows (several 256-row stripes, windows across stripe boundaries) in the
    stripe-chained layout and in group mode (G = 4: 32-row stripes)."""
    rng = np.random.default_rng(zlib.crc32(f"enum-long/{locality}".encode()))
    n = 10
    pairs = [(rng.integers(0, 2, size=int(rng.integers(513, 801))).astype(np.uint32),
              rng.integers(0, 2, size=int(rng.integers(20, 90))).astype(np.uint32)) for _ in range(n)]
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    for mode in ("units", "G4"):
        with monkeypatch.context() as m:
            if mode == "units":
                m.setenv("PA_DP_MODE", "units")
            else:
                m.setenv("PA_GROUP_WIDTH", "4")
            solver, its, ln, *_ = _solve(gpu_alg, pairs, locality, Gap("affine", 2.0, 1.0), "maximize", True, table)
            _compare_with_host(gpu_alg, its, ln, 12)


def test_small_stacks_and_seed_lists_retry(monkeypatch, gpu_alg):
    """A search stack of 1 entry and a seed list of 1 cell per lane: every lane that needs
    more is enumerated again with more room, with the same results."""
    rng = np.random.default_rng(31)
    pairs = _pairs(rng, 30)
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    for locality in ("local", "global"):
        solver, its, ln, *_ = _solve(gpu_alg, pairs, locality, Gap("affine", 2.0, 1.0), "maximize", True, table)
        want = _compare_with_host(gpu_alg, its, ln, 25)
        with monkeypatch.context() as m:
            m.setenv("PA_ENUM_STACK", "1")
            m.setenv("PA_ENUM_SEEDS", "1")
            got = gpu_alg.FirstAlignments(its[0]._res, 25, with_paths=True)
        assert np.array_equal(got.counts, want.counts)
        assert np.array_equal(got.maps, want.maps)
        assert np.array_equal(got.plen, want.plen)
        for lane in range(len(pairs)):
            for j in range(int(got.counts[lane])):
                assert np.array_equal(got.alignment(lane, j)[1], want.alignment(lane, j)[1]), (locality, lane, j)


@pytest.mark.parametrize("first", ["3", "101"])
def test_python_iterators_resume_after_device_results(monkeypatch, gpu_alg, oracle_alg, first):
    """AlignmentIterator / SolutionIterator serve the device's first results and then resume
    the host search after them: the whole sequence equals the oracle's iterators."""
    monkeypatch.setenv("PA_ENUM_FIRST", first)
    rng = np.random.default_rng(77 + int(first))
    pairs = _pairs(rng, 20, 1, 14)
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    for locality in ("local", "global"):
        o = dict(options(gpu_alg, locality=locality, count="all", gap=Gap("affine", 2.0, 1.0)), batch_size=n,
                 batch=True)
        cap = (a.shape[1], b.shape[1])
        gs = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o))
        os_ = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o))
        for kind in ("alignment", "solution"):
            its = getattr(gs, f"solve_indexed_for_{kind}_iterator")(a, b, table, ln)
            oits = getattr(os_, f"solve_indexed_for_{kind}_iterator")(a, b, table, ln)
            for lane in range(n):
                for j in range(200):
                    x, y = its[lane].next(), oits[lane].next()
                    assert (x is None) == (y is None), (locality, kind, lane, j)
                    if x is None:
                        break
                    assert x.score == y.score, (locality, kind, lane, j)
                    if kind == "alignment":
                        assert np.array_equal(np.asarray(x.s_to_t), np.asarray(y.s_to_t)), (locality, lane, j)
                    else:
                        assert np.array_equal(np.asarray(x.path), np.asarray(y.path)), (locality, lane, j)


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_alignment_codomain_of_all_optimal_solver(gpu_alg, oracle_alg, locality):
    """solve_*_for_alignment on an all-optimal solver returns each lane's first alignment of
    the search (taken from one device enumeration of every lane) with the lane's score, as
    the oracle's same call does."""
    rng = np.random.default_rng(zlib.crc32(f"first-alignment/{locality}".encode()))
    pairs = _pairs(rng, 40)
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    o = dict(options(gpu_alg, locality=locality, count="all", gap=Gap("affine", 2.0, 1.0)), batch_size=n, batch=True)
    cap = (a.shape[1], b.shape[1])
    gs = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o))
    os_ = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o))
    got = gs.solve_indexed_for_alignment(a, b, table, ln)
    want = os_.solve_indexed_for_alignment(a, b, table, ln)
    for k in range(n):
        assert got[k].score == want[k].score, (k, got[k].score, want[k].score)
        assert np.array_equal(np.asarray(got[k].s_to_t), np.asarray(want[k].s_to_t)), k
        assert np.array_equal(np.asarray(got[k].t_to_s), np.asarray(want[k].t_to_s)), k


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_solution_codomain_of_all_optimal_solver(gpu_alg, oracle_alg, locality):
    """solve_*_for_solution on an all-optimal solver: each Solution's path, alignment and
    score (the lane's first result of the search, from the device enumeration) equal the
    oracle's."""
    rng = np.random.default_rng(zlib.crc32(f"first-solution/{locality}".encode()))
    pairs = _pairs(rng, 30)
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = np.array([[2.0, -1.0], [-1.0, 2.0]], np.float32)
    o = dict(options(gpu_alg, locality=locality, detail="solution", count="all", gap=Gap("affine", 2.0, 1.0)),
             batch_size=n, batch=True)
    cap = (a.shape[1], b.shape[1])
    gs = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o))
    os_ = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o))
    got = gs.solve_indexed_for_solution(a, b, table, ln)
    want = os_.solve_indexed_for_solution(a, b, table, ln)
    for k in range(n):
        assert got[k].score == want[k].score, (k, got[k].score, want[k].score)
        gp, wp = got[k].path, want[k].path
        assert (gp is None) == (wp is None), k
        if gp is not None:
            assert np.array_equal(np.asarray(gp), np.asarray(wp)), k
        ga, wa = got[k].alignment, want[k].alignment
        assert (ga is None) == (wa is None), k
        if ga is not None:
            assert np.array_equal(np.asarray(ga.s_to_t), np.asarray(wa.s_to_t)), k
