"""The stripe-chained DP mode against the oracle (needs a GPU).

In the stripe-chained mode every 256-row stripe of a pair is a separate work ticket: the
warp that takes stripe q reads the boundary row of stripe q - 1 while another warp is still
producing it, column by column, behind a release/acquire progress counter, and the seed of
the stripes above (local optimum, semiglobal last-column optimum) travels down the chain.
The solver picks the mode for launches of few long pairs; PA_DP_MODE=units forces it here
on pairs short enough for the oracle, so every gap cost, locality and codomain of the
chained path is compared with the oracle bit for bit, including empty pairs and pairs whose
t is empty while s spans several stripes.
"""

import zlib

import numpy as np
import pytest

from _cases import Gap, call, compare, dense_of, options, pack, random_pairs

pytestmark = pytest.mark.gpu

GAPS = {"linear": Gap("linear", 2.0), "affine": Gap("affine", 5.0, 2.0)}


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


@pytest.fixture()
def chained(monkeypatch):
    monkeypatch.setenv("PA_DP_MODE", "units")


def _run_both(gpu_alg, oracle_alg, opts, method, form, pairs, table=None, eq=1.0, ne=-1.0, iter_cap=40):
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    cap = (max(a.shape[1], 1), max(b.shape[1], 1))
    sim = dense_of(a, b, ln, table) if form == "dense" else None
    o = dict(opts, batch_size=n, batch=True)
    _, g = call(gpu_alg, o, cap, method, form, a, b, ln, table=table, eq=eq, ne=ne, sim=sim)
    _, r = call(oracle_alg, o, cap, method, form, a, b, ln, table=table, eq=eq, ne=ne, sim=sim)
    return compare(method, g, r, n, iter_cap=iter_cap)


def _pairs(rng, n, lo, hi, alphabet=4):
    pairs = random_pairs(rng, n, lo, hi, alphabet=alphabet, related=0.7)
    pairs[0] = (pairs[0][0][:0], pairs[0][1])                    # empty s
    pairs[1] = (pairs[1][0], pairs[1][1][:0])                    # empty t, s over several stripes
    pairs[2] = (pairs[2][0][:700], pairs[2][1][:1])              # one column
    pairs[3] = (pairs[3][0][:256], pairs[3][1])                  # exactly one stripe
    pairs[4] = (pairs[4][0][:257], pairs[4][1])                  # one row into the second
    return pairs


def _ftable(rng, A):
    t = rng.normal(size=(A, A)).astype(np.float32)
    return ((t + t.T) / 2).astype(np.float32)


@pytest.mark.parametrize("gap", ["linear", "affine"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("method", ["score", "alignment", "solution"])
def test_chained_parity(chained, gpu_alg, oracle_alg, gap, locality, method):
    rng = np.random.default_rng(zlib.crc32(f"chain/{gap}/{locality}/{method}".encode()))
    pairs = _pairs(rng, 10, 300, 800)
    detail = "score" if method == "score" else ("solution" if method == "solution" else "alignment")
    opts = options(gpu_alg, locality=locality, detail=detail, gap=GAPS[gap])
    d = _run_both(gpu_alg, oracle_alg, opts, method, "binary", pairs, eq=2.0, ne=-3.0)
    assert d is None, f"binary: {d}"
    d = _run_both(gpu_alg, oracle_alg, opts, method, "indexed", pairs, table=_ftable(rng, 4))
    assert d is None, f"float table: {d}"
    mopts = options(gpu_alg, locality=locality, direction="minimize", detail=detail, gap=GAPS[gap])
    d = _run_both(gpu_alg, oracle_alg, mopts, method, "binary", pairs, eq=-1.0, ne=2.0)
    assert d is None, f"minimize: {d}"


@pytest.mark.parametrize("method", ["score", "alignment"])
def test_chained_dtw(chained, gpu_alg, oracle_alg, method):
    rng = np.random.default_rng(91)
    pairs = _pairs(rng, 8, 300, 700, alphabet=6)
    opts = options(gpu_alg, dtw=True, direction="minimize",
                   detail="score" if method == "score" else "alignment")
    table = np.abs(np.subtract.outer(np.arange(6.0), np.arange(6.0))).astype(np.float32)
    d = _run_both(gpu_alg, oracle_alg, opts, method, "indexed", pairs, table=table)
    assert d is None, d
    d = _run_both(gpu_alg, oracle_alg, opts, method, "dense", pairs, table=table)
    assert d is None, f"dense: {d}"


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_chained_all_optimal(chained, gpu_alg, oracle_alg, locality):
    """All-optimal masks from chained stripes: enumeration order with dedup, first 40."""
    rng = np.random.default_rng(17 + len(locality))
    pairs = random_pairs(rng, 5, 300, 600, alphabet=3, related=0.8)
    opts = options(gpu_alg, locality=locality, detail="alignment", count="all", gap=GAPS["affine"])
    d = _run_both(gpu_alg, oracle_alg, opts, "alignment_iterator", "binary", pairs, eq=1.0, ne=-1.0)
    assert d is None, d


@pytest.mark.parametrize("locality", ["local", "semiglobal"])
def test_chained_matches_group_mode_large(gpu_alg, monkeypatch, locality):
    """48 pairs of up to 2500 x 4000 (10 stripes), 20 letters, affine 10/1, int32 scoring:
    both modes, both codomains' scores and the local/semiglobal seeds, GPU against GPU."""
    rng = np.random.default_rng(33)
    n = 48
    ls = rng.integers(1, 2500, size=n)
    lt = rng.integers(1, 4000, size=n)
    a = np.zeros((n, 2500), np.uint32)
    b = np.zeros((n, 4000), np.uint32)
    for k in range(n):
        a[k, :ls[k]] = rng.integers(0, 20, size=ls[k])
        b[k, :lt[k]] = rng.integers(0, 20, size=lt[k])
    m = rng.integers(-4, 3, size=(20, 20))
    m = np.triu(m, 1) + np.triu(m, 1).T
    np.fill_diagonal(m, rng.integers(4, 12, size=20))
    table = m.astype(np.float32)
    ln = np.stack([ls, lt]).astype(np.uint16)
    out = {}
    for mode in ("groups", "units"):
        monkeypatch.setenv("PA_DP_MODE", mode)
        for detail in ("score", "alignment"):
            opts = options(gpu_alg, locality=locality, detail=detail, gap=Gap("affine", 10.0, 1.0),
                           batch_size=n)
            solver = gpu_alg.m16.create_solver(2500, 4000, gpu_alg.m16.create_options(opts))
            if detail == "score":
                out[(mode, detail)] = np.asarray(solver.solve_indexed_for_score(a, b, table, ln))
            else:
                res = solver.solve_indexed_for_alignment(a, b, table, ln)
                out[(mode, detail)] = [(r.score, r.s_to_t.tolist()) for r in res]
    assert np.array_equal(out[("groups", "score")], out[("units", "score")])
    assert out[("groups", "alignment")] == out[("units", "alignment")]


def test_autotuned_plan_matches_analytic_plan(gpu_alg, monkeypatch):
    """The autotuner times the group widths and the chained mode on the first call with a
    new workload signature; whichever it keeps, scores and alignments are those of the
    analytic plan (PA_TUNE=0)."""
    rng = np.random.default_rng(71)
    n = 1536
    ls = rng.integers(100, 700, size=n)
    lt = rng.integers(100, 700, size=n)
    a = np.zeros((n, 700), np.uint32)
    b = np.zeros((n, 700), np.uint32)
    for k in range(n):
        a[k, :ls[k]] = rng.integers(0, 4, size=ls[k])
        b[k, :lt[k]] = rng.integers(0, 4, size=lt[k])
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    ln = np.stack([ls, lt]).astype(np.uint16)
    out = {}
    for tune in ("0", "1"):
        monkeypatch.setenv("PA_TUNE", tune)
        opts = options(gpu_alg, locality="local", detail="alignment", gap=GAPS["affine"], batch_size=n)
        solver = gpu_alg.m16.create_solver(700, 700, gpu_alg.m16.create_options(opts))
        res = solver.solve_indexed_for_alignment(a, b, table, ln)
        out[tune] = [(r.score, r.s_to_t.tolist()) for r in res]
    assert out["0"] == out["1"]


def test_chained_matches_oracle_at_bench_size(gpu_alg, oracle_alg):
    """The long-pair workload at its full size: 256 pairs of 5000 x 10000 residues, 20
    letters with Dirichlet(1) frequencies, a seeded symmetric integer matrix, semiglobal
    affine 10/1, score only -- the solver's own plan (stripe-chained) over the whole bag, and
    the first pairs' scores against the oracle's two-row score (same float32 operations),
    bit for bit."""
    import bench
    a, b, ls, lt, table = bench.make_semiglobal_long(2024)
    n = a.shape[0]
    opts = dict(options(gpu_alg, locality="semiglobal", detail="score", gap=Gap("affine", 10.0, 1.0)),
                batch_size=n, batch=True)
    solver = gpu_alg.m16.create_solver(a.shape[1], b.shape[1], gpu_alg.m16.create_options(opts))
    g = np.asarray(solver.solve_indexed_for_score(a, b, table, np.stack([ls, lt]).astype(np.uint16)))
    assert solver.last_plan()["kernel"] == "stripe-chained", solver.last_plan()
    k = 6
    osol = oracle_alg.m16.create_solver(a.shape[1], b.shape[1], oracle_alg.m16.create_options(opts))
    r, _ = oracle_alg.batch_scores_lean(osol, a[:k], b[:k], table, ls[:k], lt[:k])
    assert np.array_equal(g[:k], r), (g[:k], r)
