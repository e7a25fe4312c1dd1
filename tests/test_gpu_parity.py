"""GPU results against the oracle and the reference's golden vectors (needs a GB300).

Every test calls the CUDA library through its C ABI (via pyalign_gb300.algorithm, the
drop-in for pyalign's native module) and compares with the CPU oracle on the same
seeded inputs: scores bit-exact (float32 equality, both for integer and for float
scoring, since the kernels repeat the reference's float operations), alignments,
the full enumeration order of all optimal alignments, and Solution arrays.
"""

import zlib

import numpy as np
import pytest

from _cases import Gap, call, compare, dense_of, options, pack, random_pairs
from _replay import drain, edges_of, load_golden, make_options, repack, call_args

pytestmark = pytest.mark.gpu

GOLDEN = load_golden()


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


# ---------------------------------------------------------------- golden vectors

@pytest.mark.parametrize("check", GOLDEN["checks"],
                         ids=lambda c: f'{c["test"].split(".")[-1]}-call{c["call"]}-lane{c["lane"]}')
def test_reference_known_answers(gpu_alg, check):
    """The reference's own test expectations (pyalign/tests/*.py), checked as test.py:24-34."""
    call_rec = GOLDEN["calls"][check["call"]]
    mod = gpu_alg.m16 if call_rec["index_bits"] == 16 else gpu_alg.m32
    solver = mod.create_solver(call_rec["cap"][0], call_rec["cap"][1],
                               mod.create_options(make_options(gpu_alg, call_rec["options"])))
    packed, n = repack(call_rec, solver.batch_size)
    res = getattr(solver, call_rec["method"])(*call_args(call_rec["method"], packed))
    item = res[check["lane"]]
    items = drain(item) if call_rec["method"].endswith("alignment_iterator") else [item]
    for x in items:
        assert round(abs(x.score - check["score"]), check["places"]) == 0
    assert sorted(edges_of(x) for x in items) == sorted(check["edges"])


@pytest.mark.parametrize("rec", GOLDEN["calls"], ids=lambda c: f'call{c["id"]}-{c["method"]}')
def test_reference_calls_enumeration_order(gpu_alg, rec):
    """Every recorded native call: same results in the same order as the oracle's record."""
    mod = gpu_alg.m16 if rec["index_bits"] == 16 else gpu_alg.m32
    solver = mod.create_solver(rec["cap"][0], rec["cap"][1],
                               mod.create_options(make_options(gpu_alg, rec["options"])))
    packed, n = repack(rec, solver.batch_size)
    res = getattr(solver, rec["method"])(*call_args(rec["method"], packed))
    want = rec["result"]
    if rec["method"].endswith("for_score"):
        assert np.array_equal(np.asarray(res[:n], dtype=np.float64), np.asarray(want["scores"][:n]))
        return
    for k in range(n):
        if rec["method"].endswith("alignment_iterator"):
            got = [(a.score, a.s_to_t.tolist()) for a in drain(res[k])]
            exp = [(x["score"], x["s_to_t"]) for x in want["lanes"][k]]
            assert got == exp, (k, got, exp)
        elif rec["method"].endswith("for_alignment"):
            assert res[k].score == want["lanes"][k]["score"]
            assert res[k].s_to_t.tolist() == want["lanes"][k]["s_to_t"]


# ---------------------------------------------------------------- random parity

GAPS = {
    "linear": Gap("linear", 2.0),
    "affine": Gap("affine", 5.0, 2.0),
    "general": Gap("log", 3.0, 1.0),
}
METHODS = ["score", "alignment", "alignment_iterator", "solution", "solution_iterator"]


def _run_both(gpu_alg, oracle_alg, opts, method, form, pairs, table=None, eq=1.0, ne=-1.0, bits=16,
              iter_cap=60):
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    cap = (max(a.shape[1], 1), max(b.shape[1], 1))
    sim = dense_of(a, b, ln, table) if form == "dense" else None
    o = dict(opts, batch_size=n, batch=True)
    _, g = call(gpu_alg, o, cap, method, form, a, b, ln, table=table, eq=eq, ne=ne, sim=sim, bits=bits)
    _, r = call(oracle_alg, o, cap, method, form, a, b, ln, table=table, eq=eq, ne=ne, sim=sim, bits=bits)
    return compare(method, g, r, n, iter_cap=iter_cap)


def _table(rng, A, integer=True):
    if integer:
        t = rng.integers(-4, 6, size=(A, A)).astype(np.float32)
        t = np.triu(t) + np.triu(t, 1).T
        np.fill_diagonal(t, rng.integers(2, 8, size=A))
        return t.astype(np.float32)
    t = rng.normal(size=(A, A)).astype(np.float32)
    return ((t + t.T) / 2).astype(np.float32)


@pytest.mark.parametrize("gap", ["linear", "affine", "general"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("direction", ["maximize", "minimize"])
@pytest.mark.parametrize("method", METHODS)
def test_small_parity_all_modes(gpu_alg, oracle_alg, gap, locality, direction, method):
    """Lengths 0..24 (empty and ragged pairs included), all three input forms."""
    seed = zlib.crc32(f"{gap}/{locality}/{direction}/{method}".encode())
    rng = np.random.default_rng(seed)
    count = "all" if method.endswith("iterator") else "one"
    detail = "score" if method == "score" else ("solution" if "solution" in method else "alignment")
    opts = options(gpu_alg, locality=locality, direction=direction, detail=detail, count=count,
                   gap=GAPS[gap])
    pairs = random_pairs(rng, 12, 0, 24, alphabet=4)
    pairs[0] = (pairs[0][0][:0], pairs[0][1])       # empty s
    pairs[1] = (pairs[1][0], pairs[1][1][:0])       # empty t
    pairs[2] = (pairs[2][0][:0], pairs[2][1][:0])   # both empty
    table = _table(rng, 4)
    for form in ("binary", "indexed", "dense"):
        d = _run_both(gpu_alg, oracle_alg, opts, method, form, pairs, table=table, eq=2.0, ne=-3.0)
        assert d is None, f"{form}: {d}"


@pytest.mark.parametrize("direction", ["maximize", "minimize"])
@pytest.mark.parametrize("method", METHODS)
def test_dtw_parity(gpu_alg, oracle_alg, direction, method):
    rng = np.random.default_rng(7 + METHODS.index(method))
    opts = options(gpu_alg, dtw=True, direction=direction,
                   detail="score" if method == "score" else "alignment")
    pairs = random_pairs(rng, 10, 1, 30, alphabet=6)
    table = np.abs(np.subtract.outer(np.arange(6.0), np.arange(6.0))).astype(np.float32)
    for form in ("binary", "indexed", "dense"):
        d = _run_both(gpu_alg, oracle_alg, opts, method, form, pairs, table=table, eq=0.0, ne=1.5)
        assert d is None, f"{form}: {d}"


@pytest.mark.parametrize("gap", ["linear", "affine"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("lengths", [(50, 130), (200, 700)])
def test_multi_stripe_parity(gpu_alg, oracle_alg, gap, locality, lengths):
    """Several stripes per pair, groups of 16 and 32 lanes, integer and float scoring."""
    rng = np.random.default_rng(lengths[1] + len(locality))
    pairs = random_pairs(rng, 16, lengths[0], lengths[1], alphabet=4, related=0.7)
    opts = options(gpu_alg, locality=locality, detail="alignment", gap=GAPS[gap])
    table = _table(rng, 4)
    for form in ("binary", "indexed"):
        d = _run_both(gpu_alg, oracle_alg, opts, "alignment", form, pairs, table=table, eq=2.0, ne=-3.0)
        assert d is None, f"{form}: {d}"
    ftable = _table(rng, 4, integer=False)
    d = _run_both(gpu_alg, oracle_alg, opts, "alignment", "indexed", pairs, table=ftable)
    assert d is None, f"float table: {d}"
    d = _run_both(gpu_alg, oracle_alg, dict(opts, codomain=opts["codomain"]), "score", "dense", pairs,
                  table=ftable)
    assert d is None, f"dense: {d}"


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_all_optimal_long(gpu_alg, oracle_alg, locality):
    """All-optimal enumeration order with dedup on multi-stripe pairs (first 40 results)."""
    rng = np.random.default_rng(11)
    pairs = random_pairs(rng, 6, 100, 300, alphabet=3, related=0.8)
    opts = options(gpu_alg, locality=locality, detail="alignment", count="all", gap=GAPS["affine"])
    d = _run_both(gpu_alg, oracle_alg, opts, "alignment_iterator", "binary", pairs, eq=1.0, ne=-1.0,
                  iter_cap=40)
    assert d is None, d


def test_m32_and_return_dup(gpu_alg, oracle_alg):
    rng = np.random.default_rng(3)
    pairs = random_pairs(rng, 8, 5, 40, alphabet=2)
    opts = options(gpu_alg, locality="local", detail="alignment", count="all", gap=GAPS["linear"],
                   return_dup=True)
    d = _run_both(gpu_alg, oracle_alg, opts, "alignment_iterator", "binary", pairs, bits=32, iter_cap=30)
    assert d is None, d


def test_errors_match_reference(gpu_alg):
    opts = options(gpu_alg, detail="alignment", gap=GAPS["linear"], batch=True, batch_size=4)
    mod = gpu_alg.m16
    s = mod.create_solver(8, 8, mod.create_options(opts))
    a = np.zeros((4, 8), np.uint32)
    ln = np.full((2, 4), 8, np.uint16)
    table = np.eye(3, dtype=np.float32)
    a[1, 3] = 5
    with pytest.raises(ValueError, match="out of bounds index in a"):
        s.solve_indexed_for_alignment(a, np.zeros((4, 8), np.uint32), table, ln)
    with pytest.raises(ValueError, match="batch size"):
        s.solve_binary_for_score(np.zeros((3, 8), np.uint32), np.zeros((3, 8), np.uint32), 1, -1,
                                 np.full((2, 3), 8, np.uint16))
    with pytest.raises(RuntimeError, match="exceeds configured maximum length"):
        s.solve_binary_for_score(np.zeros((4, 9), np.uint32), np.zeros((4, 8), np.uint32), 1, -1, ln)


def test_bag_at_once_batch_form(gpu_alg, oracle_alg):
    """pa_solve_batch (the ProblemBatch throughput path) against the oracle, uneven lengths."""
    import ctypes
    rng = np.random.default_rng(5)
    pairs = random_pairs(rng, 300, 20, 400, alphabet=4, related=0.5)
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    opts = options(gpu_alg, locality="local", detail="alignment", gap=Gap("affine", 5.0, 2.0), batch_size=n)
    mod = gpu_alg.m16
    solver = mod.create_solver(a.shape[1], b.shape[1], mod.create_options(opts))
    L = gpu_alg.lib()
    ln32 = np.ascontiguousarray(ln, dtype=np.int32)
    sizes = np.minimum(ln[0], ln[1]).astype(np.int64)
    offs = np.zeros(n, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    maps = np.full(int(sizes.sum()), -7, np.int32)
    scores = np.zeros(n, np.float32)
    bt = gpu_alg.Batch(form=1, location=0, batch=n, n_s=a.shape[1], n_t=b.shape[1],
                       a=a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                       b=b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                       table=table.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), table_rows=4, table_cols=4,
                       length=ln32.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    gpu_alg.check(L.pa_solve_batch(solver.handle, ctypes.byref(bt), scores.ctypes.data, maps.ctypes.data,
                                   offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
    _, ref = call(oracle_alg, dict(opts, batch=True), (a.shape[1], b.shape[1]), "alignment", "indexed", a, b, ln,
                  table=table)
    for k in range(n):
        assert scores[k] == ref[k].score, k
        want = ref[k].s_to_t if ln[0, k] <= ln[1, k] else ref[k].t_to_s
        assert np.array_equal(maps[offs[k]:offs[k] + sizes[k]], want), k


@pytest.mark.parametrize("subst", ["profile", "table"])
@pytest.mark.parametrize("gap", ["linear", "affine"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_twenty_letter_table(gpu_alg, oracle_alg, monkeypatch, subst, gap, locality):
    """A 20-letter integer table: read through the per-letter int8 profile in shared memory
    (the default for integer tables of up to 32 letters) and through plain table lookups."""
    if subst == "table":
        monkeypatch.setenv("PA_SUBST", "table")
    rng = np.random.default_rng(zlib.crc32(f"twenty/{gap}/{locality}".encode()))
    m = rng.integers(-4, 3, size=(20, 20))
    m = np.triu(m, 1) + np.triu(m, 1).T
    np.fill_diagonal(m, rng.integers(4, 12, size=20))
    table = m.astype(np.float32)
    pairs = random_pairs(rng, 12, 0, 300, alphabet=20, related=0.6)
    for method, count in (("alignment", "one"), ("score", "one"), ("alignment_iterator", "all")):
        opts = options(gpu_alg, locality=locality, detail="score" if method == "score" else "alignment",
                       count=count, gap=GAPS[gap])
        d = _run_both(gpu_alg, oracle_alg, opts, method, "indexed", pairs, table=table, iter_cap=20)
        assert d is None, f"{method}: {d}"
        mopts = options(gpu_alg, locality=locality, direction="minimize",
                        detail="score" if method == "score" else "alignment", count=count, gap=GAPS[gap])
        d = _run_both(gpu_alg, oracle_alg, mopts, method, "indexed", pairs, table=-table, iter_cap=20)
        assert d is None, f"minimize {method}: {d}"


@pytest.mark.parametrize("gap", ["linear", "affine", "dtw"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_one_and_two_column_kernels(gpu_alg, oracle_alg, monkeypatch, gap, locality):
    """Integer scoring runs the two-column kernel (a lane updates columns j and j + 1 per
    step) by default; PA_DP_COLS=1 selects the one-column kernel.  Both against the oracle,
    odd and even |t|, several stripes, score and one traceback."""
    if gap == "dtw" and locality != "global":
        pytest.skip("DTW is global")
    rng = np.random.default_rng(zlib.crc32(f"cols/{gap}/{locality}".encode()))
    pairs = random_pairs(rng, 14, 0, 300, alphabet=4, related=0.6)
    pairs[0] = (pairs[0][0][:1], pairs[0][1][:1])
    pairs[1] = (pairs[1][0][:257], pairs[1][1][:3])
    for cols in ("1", "2"):
        monkeypatch.setenv("PA_DP_COLS", cols)
        for method in ("score", "alignment"):
            if gap == "dtw":
                opts = options(gpu_alg, dtw=True, direction="minimize",
                               detail="score" if method == "score" else "alignment")
                table = np.abs(np.subtract.outer(np.arange(4.0), np.arange(4.0))).astype(np.float32)
            else:
                opts = options(gpu_alg, locality=locality, detail="score" if method == "score" else "alignment",
                               gap=GAPS[gap])
                table = _table(rng, 4)
            d = _run_both(gpu_alg, oracle_alg, opts, method, "indexed", pairs, table=table)
            assert d is None, f"cols={cols} {method}: {d}"
            if gap != "dtw":
                d = _run_both(gpu_alg, oracle_alg, opts, method, "binary", pairs, eq=2.0, ne=-3.0)
                assert d is None, f"cols={cols} binary {method}: {d}"


@pytest.mark.parametrize("width", ["1", "2"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_lane_per_pair_widths(gpu_alg, oracle_alg, monkeypatch, width, locality):
    """Group widths below four lanes (1: a lane per pair, its 8 rows per stripe) that the
    autotuner offers for short pairs; integer and float scoring against the oracle."""
    monkeypatch.setenv("PA_GROUP_WIDTH", width)
    rng = np.random.default_rng(zlib.crc32(f"narrow/{width}/{locality}".encode()))
    pairs = random_pairs(rng, 40, 0, 60, alphabet=4, related=0.6)
    for method in ("score", "alignment", "solution"):
        detail = "score" if method == "score" else ("solution" if method == "solution" else "alignment")
        opts = options(gpu_alg, locality=locality, detail=detail, gap=GAPS["affine"])
        d = _run_both(gpu_alg, oracle_alg, opts, method, "binary", pairs, eq=2.0, ne=-3.0)
        assert d is None, f"{method}: {d}"
        d = _run_both(gpu_alg, oracle_alg, opts, method, "indexed", pairs, table=_table(rng, 4, integer=False))
        assert d is None, f"float {method}: {d}"
    opts = options(gpu_alg, locality=locality, detail="alignment", count="all", gap=GAPS["linear"])
    d = _run_both(gpu_alg, oracle_alg, opts, "alignment_iterator", "binary", pairs[:12], eq=1.0, ne=-1.0, iter_cap=20)
    assert d is None, f"all optimal: {d}"
