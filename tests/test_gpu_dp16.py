"""The packed 16-bit twin-pair DP kernel against the oracle (needs a GPU).

The solver runs two pairs per lane in the two 16-bit halves of every register whenever a
launch's value bounds fit 16 bits (indexed form, at most 4 letters of t, similarities in
[-8, 7], gap costs >= 1, local or global, one traceback or none).  Here every such case is
compared with the oracle bit for bit: ragged twins (the two pairs of a twin differ in |s|
and |t|), empty pairs, single rows and columns, stripe-multiple lengths, an odd pair count
(the last twin has one pair), all-mismatch pairs whose local optimum is 0, several group
widths, maximize and minimize.  The kernel family that ran is read back from the solver, and
launches outside the bounds must fall back to the int32 kernels.  A bench-like bag is
compared with the int32 kernels GPU against GPU.
"""

import zlib

import numpy as np
import pytest

from _cases import Gap, call, compare, options, pack, random_pairs

pytestmark = pytest.mark.gpu

GAPS = {"linear": Gap("linear", 2.0), "affine": Gap("affine", 5.0, 2.0)}
TWINS = {"1": "16-bit twins", "2": "16-bit twins, two-column", "blk": "16-bit twins, 4x4 blocks"}


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


@pytest.fixture()
def analytic(monkeypatch):
    """The analytic plan in group mode (few-pair launches would otherwise be stripe-chained)."""
    monkeypatch.setenv("PA_TUNE", "0")
    monkeypatch.setenv("PA_DP_MODE", "groups")


@pytest.fixture(params=["1", "2", "blk"])
def cols(request, monkeypatch):
    """One or two columns per lane step of 8 rows, or 4 x 4 blocks (4 rows, 4 columns)."""
    if request.param == "1":
        monkeypatch.setenv("PA_DP_COLS", "1")
    if request.param == "blk":
        monkeypatch.setenv("PA_DP_BLOCK", "1")
    return request.param


def _table(rng, direction):
    t = rng.integers(-4, 0, size=(4, 4)).astype(np.float32)
    np.fill_diagonal(t, rng.integers(2, 7, size=4))
    return -t if direction == "minimize" else t


def _pairs(rng, n):
    pairs = random_pairs(rng, n, 1, 300, alphabet=4, related=0.6)
    pairs[0] = (pairs[0][0][:0], pairs[0][1])                 # empty s
    pairs[1] = (pairs[1][0], pairs[1][1][:0])                 # empty t
    pairs[2] = (pairs[2][0][:1], pairs[2][1])                 # one row
    pairs[3] = (pairs[3][0], pairs[3][1][:1])                 # one column
    pairs[4] = (pairs[4][0][:64], pairs[4][1][:64])           # one stripe of G = 8 exactly
    pairs[5] = (pairs[5][0][:65], pairs[5][1])                # one row into the next stripe
    pairs[6] = (np.zeros(40, np.uint32), np.ones(37, np.uint32))   # all mismatches: optimum 0
    pairs[7] = (np.zeros(9, np.uint32), np.zeros(250, np.uint32))  # twin partner of very different shape
    return pairs


def _run(gpu_alg, oracle_alg, opts, method, pairs, table):
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    cap = (max(a.shape[1], 1), max(b.shape[1], 1))
    o = dict(opts, batch_size=n, batch=True)
    solver, g = call(gpu_alg, o, cap, method, "indexed", a, b, ln, table=table)
    plan = solver.last_plan()
    _, r = call(oracle_alg, o, cap, method, "indexed", a, b, ln, table=table)
    return plan, compare(method, g, r, n)


@pytest.mark.parametrize("gap", ["linear", "affine"])
@pytest.mark.parametrize("locality", ["local", "global"])
@pytest.mark.parametrize("method", ["score", "alignment"])
@pytest.mark.parametrize("direction", ["maximize", "minimize"])
def test_dp16_parity(analytic, cols, gpu_alg, oracle_alg, gap, locality, method, direction):
    rng = np.random.default_rng(zlib.crc32(f"dp16/{gap}/{locality}/{method}/{direction}".encode()))
    pairs = _pairs(rng, 61)
    detail = "score" if method == "score" else "alignment"
    opts = options(gpu_alg, locality=locality, direction=direction, detail=detail, gap=GAPS[gap])
    plan, d = _run(gpu_alg, oracle_alg, opts, method, pairs, _table(rng, direction))
    assert plan["kernel"] == TWINS[cols], plan
    assert d is None, d


@pytest.mark.parametrize("G", ["1", "2", "4", "16", "32"])
def test_dp16_group_widths(monkeypatch, cols, gpu_alg, oracle_alg, G):
    monkeypatch.setenv("PA_GROUP_WIDTH", G)
    rng = np.random.default_rng(int(G) + 500)
    pairs = _pairs(rng, 45)
    opts = options(gpu_alg, locality="local", detail="alignment", gap=GAPS["affine"])
    plan, d = _run(gpu_alg, oracle_alg, opts, "alignment", pairs, _table(rng, "maximize"))
    assert plan["kernel"] == TWINS[cols] and plan["G"] == int(G), plan
    assert d is None, d


@pytest.mark.parametrize("widths", ["8,16,16,32", "1,4,16,2", "32,8,2,16"])
@pytest.mark.parametrize("C", ["1", "2"])
@pytest.mark.parametrize("method", ["score", "alignment"])
def test_dp16_bucket_widths(analytic, monkeypatch, gpu_alg, oracle_alg, widths, C, method):
    """A group width per length bucket of |s| (<= 128, <= 256, <= 512, longer) in one launch:
    pairs of every bucket, odd bucket sizes (a twin that would straddle two buckets takes the
    next bucket's first pair at the earlier bucket's width), empty pairs, an odd pair count."""
    monkeypatch.setenv("PA_BUCKET_WIDTHS", widths)
    if C == "1":
        monkeypatch.setenv("PA_DP_COLS", "1")
    rng = np.random.default_rng(zlib.crc32(f"buckets/{widths}/{C}/{method}".encode()))
    pairs = _pairs(rng, 30) + random_pairs(rng, 17, 129, 256, alphabet=4, related=0.6) \
        + random_pairs(rng, 9, 257, 512, alphabet=4, related=0.6) + random_pairs(rng, 7, 513, 700, alphabet=4,
                                                                                  related=0.6)
    pairs = [pairs[k] for k in rng.permutation(len(pairs))]
    detail = "score" if method == "score" else "alignment"
    opts = options(gpu_alg, locality="local", detail=detail, gap=GAPS["affine"])
    table = rng.integers(-4, 0, size=(4, 4)).astype(np.float32)  # matches +2: 16-bit bounds at |s| = 700
    np.fill_diagonal(table, 2.0)
    plan, d = _run(gpu_alg, oracle_alg, opts, method, pairs, table)
    assert plan["kernel"] == TWINS[C] and plan["bucket_widths"] == [int(g) for g in widths.split(",")], plan
    assert d is None, d
    # the 4 x 4 block kernel keeps one width
    monkeypatch.setenv("PA_DP_BLOCK", "1")
    plan, d = _run(gpu_alg, oracle_alg, opts, method, pairs, table)
    assert plan["kernel"] == TWINS["blk"] and plan["bucket_widths"] is None, plan
    assert d is None, d


def test_dp16_bounds_fall_back(analytic, gpu_alg, oracle_alg):
    """Outside the 16-bit bounds the int32 kernels run, with the same results."""
    rng = np.random.default_rng(77)
    pairs = _pairs(rng, 20)
    opts = options(gpu_alg, locality="local", detail="alignment", gap=GAPS["affine"])
    table = _table(rng, "maximize")
    table[0, 0] = 9.0                                         # similarity outside [-8, 7]
    plan, d = _run(gpu_alg, oracle_alg, opts, "alignment", pairs, table)
    assert not plan["kernel"].startswith("16-bit"), plan
    assert d is None, d
    # a local optimum that may exceed 2047: 7 * 300 > 2047
    table = np.full((4, 4), -2.0, np.float32)
    np.fill_diagonal(table, 7.0)
    long_pairs = [(np.zeros(300, np.uint32), np.zeros(300, np.uint32))] + pairs[:5]
    plan, d = _run(gpu_alg, oracle_alg, opts, "alignment", long_pairs, table)
    assert not plan["kernel"].startswith("16-bit"), plan
    assert d is None, d
    # a zero gap extension (rows past |s| would not stay below the optimum)
    opts0 = options(gpu_alg, locality="local", detail="alignment", gap=Gap("affine", 3.0, 0.0))
    plan, d = _run(gpu_alg, oracle_alg, opts0, "alignment", pairs, _table(rng, "maximize"))
    assert not plan["kernel"].startswith("16-bit"), plan
    assert d is None, d


@pytest.mark.parametrize("locality", ["local", "global"])
def test_dp16_matches_int32_large(gpu_alg, monkeypatch, cols, locality):
    """3000 pairs of |s|, |t| ~ U[100, 1000] (DNA +2/-3, affine 5/2; global only up to the
    lengths the bounds admit): scores and alignments of the 16-bit kernel equal the int32
    kernels', GPU against GPU."""
    rng = np.random.default_rng(808)
    n = 3000
    hi = 1000 if locality == "local" else 250
    ls = rng.integers(100 if locality == "local" else 20, hi + 1, size=n)
    lt = rng.integers(100 if locality == "local" else 20, hi + 1, size=n)
    a = rng.integers(0, 4, size=(n, hi)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, hi)).astype(np.uint32)
    half = n // 2
    b[:half, :hi] = a[:half, :hi]                             # related half: mutated copies
    mut = rng.random(size=(half, hi)) < 0.1
    b[:half][mut] = rng.integers(0, 4, size=int(mut.sum()))
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    ln = np.stack([ls, lt]).astype(np.uint16)
    monkeypatch.setenv("PA_TUNE", "0")
    monkeypatch.setenv("PA_DP_MODE", "groups")
    out = {}
    for dp16 in ("1", "0"):
        monkeypatch.setenv("PA_DP16", dp16)
        for detail in ("score", "alignment"):
            opts = options(gpu_alg, locality=locality, detail=detail, gap=GAPS["affine"], batch_size=n)
            solver = gpu_alg.m16.create_solver(hi, hi, gpu_alg.m16.create_options(opts))
            if detail == "score":
                out[(dp16, detail)] = np.asarray(solver.solve_indexed_for_score(a, b, table, ln))
            else:
                res = solver.solve_indexed_for_alignment(a, b, table, ln)
                out[(dp16, detail)] = [(r.score, r.s_to_t.tolist()) for r in res]
            kernel = solver.last_plan()["kernel"]
            assert (kernel == TWINS[cols]) == (dp16 == "1"), (dp16, kernel)
    assert np.array_equal(out[("1", "score")], out[("0", "score")])
    assert out[("1", "alignment")] == out[("0", "alignment")]


def test_dp16_bad_codes_then_valid(analytic, gpu_alg, oracle_alg):
    """A code outside the table raises (the kernels check the launch's code maxima and do no
    work), and the same solver then solves a valid bag correctly."""
    rng = np.random.default_rng(5150)
    pairs = _pairs(rng, 30)
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = _table(rng, "maximize")
    opts = dict(options(gpu_alg, locality="local", detail="alignment", gap=GAPS["affine"]), batch_size=n, batch=True)
    solver = gpu_alg.m16.create_solver(a.shape[1], b.shape[1], gpu_alg.m16.create_options(opts))
    bad = b.copy()
    bad[3, 0] = 4
    with pytest.raises(ValueError, match="out of bounds index in b"):
        solver.solve_indexed_for_alignment(a, bad, table, ln)
    g = solver.solve_indexed_for_alignment(a, b, table, ln)
    assert solver.last_plan()["kernel"].startswith("16-bit"), solver.last_plan()
    _, r = call(oracle_alg, opts, (a.shape[1], b.shape[1]), "alignment", "indexed", a, b, ln, table=table)
    d = compare("alignment", g, r, n)
    assert d is None, d


@pytest.mark.parametrize("plan", ["twins-G16", "blocks-G8", "blocks-G16", "buckets-8,16,16,32", "own"])
def test_dp16_matches_oracle_at_bench_shapes(gpu_alg, oracle_alg, monkeypatch, plan):
    """4,096 pairs drawn like the batched workload (DNA, |s|, |t| ~ U[100, 1000], half of them
    a query and a 10%-mutated copy; local affine 5/2, +2/-3; score + one traceback) against
    the oracle, every score and every alignment map bit for bit: with the batched
    workload's plan (the 16-bit twin kernel, two columns per step, G = 16), with the block
    kernel, with a group width per length bucket, and with the plan the solver picks for
    this bag on its own."""
    import bench
    if plan.startswith("buckets"):
        monkeypatch.setenv("PA_BUCKET_WIDTHS", plan.split("-")[1])
        monkeypatch.setenv("PA_DP_MODE", "groups")          # 4,096 such pairs would run stripe-chained
    elif plan != "own":
        monkeypatch.setenv("PA_GROUP_WIDTH", plan.split("-G")[1])
    if plan.startswith("blocks"):
        monkeypatch.setenv("PA_DP_BLOCK", "1")
    a, b, ls, lt, table = bench.make_workload(4096, 4242)
    n = a.shape[0]
    opts = dict(options(gpu_alg, locality="local", detail="alignment", gap=GAPS["affine"]), batch_size=n, batch=True)
    solver = gpu_alg.m16.create_solver(a.shape[1], b.shape[1], gpu_alg.m16.create_options(opts))
    res = solver.solve_indexed_for_alignment(a, b, table, np.stack([ls, lt]).astype(np.uint16))
    if plan.startswith("buckets"):
        assert solver.last_plan()["bucket_widths"] == [8, 16, 16, 32], solver.last_plan()
    elif plan != "own":
        want = TWINS["blk"] if plan.startswith("blocks") else TWINS["2"]
        assert solver.last_plan()["kernel"] == want and solver.last_plan()["G"] == int(plan.split("-G")[1]), \
            solver.last_plan()
    osol = oracle_alg.m16.create_solver(a.shape[1], b.shape[1], oracle_alg.m16.create_options(opts))
    osc, omp, offs, _ = oracle_alg.batch_alignments(osol, a, b, table, ls, lt)
    bad = []
    for k in range(n):
        m = res[k].s_to_t if ls[k] <= lt[k] else res[k].t_to_s
        if res[k].score != osc[k] or not np.array_equal(np.asarray(m), omp[offs[k]:offs[k + 1]]):
            bad.append(k)
    assert not bad, (len(bad), bad[:10])


def test_dp16_tuned_two_length_modes(gpu_alg, oracle_alg, monkeypatch):
    """2,048 pairs in two length modes -- short queries (|s| ~ U[8, 64]) and long ones (|s| ~
    U[600, 1000]), |t| ~ U[400, 1000] for both -- solved with the plan the tuner picks
    (uniform widths, and a width per length bucket where that times faster), against the
    oracle bit for bit; a second solve of the same signature takes the tuned plan."""
    rng = np.random.default_rng(2222)
    n, hi = 2048, 1000
    ls = np.where(np.arange(n) % 2 == 0, rng.integers(8, 65, n), rng.integers(600, 1001, n))
    lt = rng.integers(400, 1001, n)
    a = rng.integers(0, 4, size=(n, hi)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, hi)).astype(np.uint32)
    b[: n // 2, :hi] = a[: n // 2, :hi]
    mut = rng.random(size=(n // 2, hi)) < 0.1
    b[: n // 2][mut] = rng.integers(0, 4, size=int(mut.sum()))
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    monkeypatch.setenv("PA_DP_MODE", "groups")
    opts = dict(options(gpu_alg, locality="local", detail="alignment", gap=GAPS["affine"]), batch_size=n, batch=True)
    ln = np.stack([ls, lt]).astype(np.uint16)
    osol = oracle_alg.m16.create_solver(hi, hi, oracle_alg.m16.create_options(opts))
    osc, omp, offs, _ = oracle_alg.batch_alignments(osol, a, b, table, ls, lt)
    plans = []
    for rep in range(2):
        solver = gpu_alg.m16.create_solver(hi, hi, gpu_alg.m16.create_options(opts))
        res = solver.solve_indexed_for_alignment(a, b, table, ln)
        plans.append(solver.last_plan())
        bad = [k for k in range(n)
               if res[k].score != osc[k] or not np.array_equal(
                   np.asarray(res[k].s_to_t if ls[k] <= lt[k] else res[k].t_to_s), omp[offs[k]:offs[k + 1]])]
        assert not bad, (rep, len(bad), bad[:10], plans[-1])
    print("tuned plan:", plans[0])
    assert plans[0]["kernel"].startswith("16-bit") and plans[0] == plans[1], plans
