"""General (Waterman-Smith-Beyer) gap costs at longer lengths against the oracle (needs a GPU).

The general-gap kernel sweeps anti-diagonals with one CTA per pair, every cell scanning its
whole column and row history (solver.h:3138-3183), and finds the seeds with a block
reduction that keeps the reference's scan order.  Pairs of up to 160 x 160 with a
logarithmic gap cost (u + v ln k), every locality, both directions, score and one
alignment: scores and alignment maps bit for bit against the oracle.
"""

import zlib

import numpy as np
import pytest

from _cases import Gap, options, pack, random_pairs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("direction", ["maximize", "minimize"])
def test_general_gap_parity_long(gpu_alg, oracle_alg, locality, direction):
    rng = np.random.default_rng(zlib.crc32(f"wsb/{locality}/{direction}".encode()))
    pairs = random_pairs(rng, 24, 60, 160, alphabet=4, related=0.6)
    pairs[0] = (pairs[0][0][:0], pairs[0][1])
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = rng.integers(-3, 4, size=(4, 4)).astype(np.float32)
    np.fill_diagonal(table, 3.0)
    if direction == "minimize":
        table = -table
    o = dict(options(gpu_alg, locality=locality, direction=direction, detail="alignment",
                     gap=Gap("log", 3.0, 1.0)), batch_size=n, batch=True)
    cap = (a.shape[1], b.shape[1])
    g = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o)).solve_indexed_for_alignment(a, b, table, ln)
    r = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o)).solve_indexed_for_alignment(
        a, b, table, ln)
    for k in range(n):
        assert g[k].score == r[k].score, (k, g[k].score, r[k].score)
        assert np.array_equal(np.asarray(g[k].s_to_t), np.asarray(r[k].s_to_t)), k


_LONG = {}


def _long_case(oracle_alg, locality):
    """Pairs whose diagonals hold more cells than a block has warps (up to 600 x 900), a
    one-letter query, an empty query; the oracle's scores and maps, computed once."""
    if locality not in _LONG:
        rng = np.random.default_rng(zlib.crc32(f"wsb-long/{locality}".encode()))
        s0 = rng.integers(0, 4, 600).astype(np.uint32)
        t0 = np.concatenate([s0[:500], rng.integers(0, 4, 400).astype(np.uint32)])
        t0[rng.random(900) < 0.1] = rng.integers(0, 4, 1)[0]
        s1 = rng.integers(0, 4, 450).astype(np.uint32)
        t1 = s1.copy()
        t1[rng.random(450) < 0.2] = 1
        pairs = [(s0, t0), (s1, t1), (s0[:1], t0[:700]), (s0[:0], t1[:300])]
        a, b, ln = pack(pairs, len(pairs))
        table = np.full((4, 4), -2.0, np.float32)
        np.fill_diagonal(table, 3.0)
        o = dict(options(oracle_alg, locality=locality, detail="alignment", gap=Gap("log", 3.0, 1.0)),
                 batch_size=len(pairs), batch=True)
        r = oracle_alg.m16.create_solver(a.shape[1], b.shape[1], oracle_alg.m16.create_options(o)) \
            .solve_indexed_for_alignment(a, b, table, ln)
        want = [(r[k].score, np.asarray(r[k].s_to_t).copy(), np.asarray(r[k].t_to_s).copy())
                for k in range(len(pairs))]
        _LONG[locality] = (a, b, ln, table, want)
    return _LONG[locality]


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("split", ["default", "one_cta", "cluster_of_2", "thread_per_cell", "two_warps"])
def test_general_gap_long_diagonals(gpu_alg, oracle_alg, monkeypatch, locality, split):
    """Diagonals of up to 600 cells: a cluster of 4 CTAs per pair (the default for 4 such
    pairs), one CTA and a cluster of 2 (PA_WSB_CLUSTER), every cell by one thread
    (PA_WSB_WARP_CELLS=0) and 64-thread blocks (PA_WSB_THREADS=64), each against the oracle
    bit for bit; the one-alignment walk runs on the device."""
    if split == "one_cta":
        monkeypatch.setenv("PA_WSB_CLUSTER", "1")
    elif split == "cluster_of_2":
        monkeypatch.setenv("PA_WSB_CLUSTER", "2")
    elif split == "thread_per_cell":
        monkeypatch.setenv("PA_WSB_WARP_CELLS", "0")
    elif split == "two_warps":
        monkeypatch.setenv("PA_WSB_THREADS", "64")
    a, b, ln, table, want = _long_case(oracle_alg, locality)
    o = dict(options(gpu_alg, locality=locality, detail="alignment", gap=Gap("log", 3.0, 1.0)),
             batch_size=len(want), batch=True)
    solver = gpu_alg.m16.create_solver(a.shape[1], b.shape[1], gpu_alg.m16.create_options(o))
    g = solver.solve_indexed_for_alignment(a, b, table, ln)
    for k, (sc, s_to_t, t_to_s) in enumerate(want):
        assert g[k].score == sc, (k, g[k].score, sc)
        assert np.array_equal(np.asarray(g[k].s_to_t), s_to_t), k
        assert np.array_equal(np.asarray(g[k].t_to_s), t_to_s), k
    scores = solver.solve_indexed_for_score(a, b, table, ln)
    assert np.array_equal(np.asarray(scores, np.float32), np.array([w[0] for w in want], np.float32))


def test_general_gap_batch_entry_writes_maps(gpu_alg, oracle_alg):
    """pa_solve_batch with general gap costs: scores and maps in the caller's host and device
    buffers equal the oracle's."""
    import ctypes
    torch = pytest.importorskip("torch")
    a, b, ln, table, want = _long_case(oracle_alg, "local")
    n = len(want)
    o = dict(options(gpu_alg, locality="local", detail="alignment", gap=Gap("log", 3.0, 1.0)), batch_size=n, batch=True)
    solver = gpu_alg.m16.create_solver(a.shape[1], b.shape[1], gpu_alg.m16.create_options(o))
    sizes = np.minimum(ln[0], ln[1]).astype(np.int64)
    offs = np.zeros(n, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    length = np.ascontiguousarray(ln, dtype=np.int32)
    want_sc = np.array([w[0] for w in want], np.float32)
    want_mp = np.concatenate([w[1] if ln[0, k] <= ln[1, k] else w[2] for k, w in enumerate(want)]).astype(np.int32)
    P = ctypes.POINTER
    L = gpu_alg.lib()
    # host buffers
    sc = np.full(n, np.nan, np.float32)
    mp = np.full(int(sizes.sum()), -7, np.int32)
    bt = gpu_alg.Batch(form=1, location=0, batch=n, n_s=a.shape[1], n_t=b.shape[1],
                       a=a.ctypes.data_as(P(ctypes.c_uint32)), b=b.ctypes.data_as(P(ctypes.c_uint32)),
                       table=table.ctypes.data_as(P(ctypes.c_float)), table_rows=4, table_cols=4,
                       length=length.ctypes.data_as(P(ctypes.c_int32)))
    gpu_alg.check(L.pa_solve_batch(solver.handle, ctypes.byref(bt), sc.ctypes.data_as(ctypes.c_void_p),
                                   mp.ctypes.data_as(ctypes.c_void_p), offs.ctypes.data_as(P(ctypes.c_int64))))
    assert np.array_equal(sc, want_sc)
    assert np.array_equal(mp, want_mp)
    # device buffers
    a_d, b_d = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    t_d = torch.from_numpy(table).cuda()
    sc_d = torch.full((n,), float("nan"), device="cuda")
    mp_d = torch.full((int(sizes.sum()),), -7, dtype=torch.int32, device="cuda")
    bt = gpu_alg.Batch(form=1, location=1, batch=n, n_s=a.shape[1], n_t=b.shape[1],
                       a=ctypes.cast(a_d.data_ptr(), P(ctypes.c_uint32)), b=ctypes.cast(b_d.data_ptr(), P(ctypes.c_uint32)),
                       table=ctypes.cast(t_d.data_ptr(), P(ctypes.c_float)), table_rows=4, table_cols=4,
                       length=length.ctypes.data_as(P(ctypes.c_int32)))
    gpu_alg.check(L.pa_solve_batch(solver.handle, ctypes.byref(bt), ctypes.c_void_p(sc_d.data_ptr()),
                                   ctypes.c_void_p(mp_d.data_ptr()), offs.ctypes.data_as(P(ctypes.c_int64))))
    torch.cuda.synchronize()
    assert np.array_equal(sc_d.cpu().numpy(), want_sc)
    assert np.array_equal(mp_d.cpu().numpy(), want_mp)


@pytest.mark.parametrize("gap", [Gap("log", 3.0, 1.0), Gap("affine", 5.0, 2.0)])
def test_alignment_results_refuse_matrix_reads(gpu_alg, gap):
    """An alignment result keeps no cell matrices (general gaps: walked on the device; other
    gaps: only the maps come back): the traceback-matrix and value reads are refused with an
    error instead of reading what was never copied."""
    import ctypes
    rng = np.random.default_rng(9)
    pairs = random_pairs(rng, 3, 20, 40, alphabet=4, related=0.5)
    a, b, ln = pack(pairs, 3)
    table = np.full((4, 4), -1.0, np.float32)
    np.fill_diagonal(table, 2.0)
    o = dict(options(gpu_alg, locality="local", detail="alignment", gap=gap), batch_size=3, batch=True)
    solver = gpu_alg.m16.create_solver(a.shape[1], b.shape[1], gpu_alg.m16.create_options(o))
    r = solver._call("alignment", "indexed", (a, b, table, ln))  # the result object of the C ABI
    L = gpu_alg.lib()
    res = r.ptr
    ls, lt = int(ln[0, 0]), int(ln[1, 0])
    buf = np.zeros(3 * (ls + 1) * (lt + 1) * 2, np.int32)
    assert L.pa_result_tb_matrix(res, 0, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) != 0
    assert L.pa_result_tb_edges(res, 0, 0, None) == -1
    vals = np.zeros(3 * (ls + 1) * (lt + 1), np.float32)
    assert L.pa_result_values(res, 0, vals.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) != 0
    mp = np.zeros(min(ls, lt), np.int32)
    assert L.pa_result_alignment(res, 0, mp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) == 0  # still usable
    assert (mp >= -1).all()


@pytest.mark.parametrize("form", ["smem_1", "global_1", "global_2", "global_4"])
@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
def test_general_gap_shared_memory_rows(gpu_alg, oracle_alg, monkeypatch, form, locality):
    """Pairs of up to 220 x 200, whose rows fit a CTA's shared memory: one CTA with the rows
    in shared memory (the default for one CTA per pair), one CTA from global memory
    (PA_WSB_SMEM=0), and clusters of 2 and 4 CTAs (global memory), each against the oracle bit
    for bit, with |s| > |t| and |s| < |t| pairs and a one-letter query."""
    kind, c = form.split("_")
    monkeypatch.setenv("PA_WSB_CLUSTER", c)
    if kind == "global":
        monkeypatch.setenv("PA_WSB_SMEM", "0")
    rng = np.random.default_rng(zlib.crc32(f"wsb-smem/{locality}".encode()))
    pairs = random_pairs(rng, 10, 90, 200, alphabet=4, related=0.7)
    pairs[1] = (rng.integers(0, 4, 220).astype(np.uint32), pairs[1][1][:57])
    pairs[2] = (pairs[2][0][:1], pairs[2][1])
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    table = rng.integers(-3, 4, size=(4, 4)).astype(np.float32)
    np.fill_diagonal(table, 3.0)
    o = dict(options(gpu_alg, locality=locality, detail="alignment", gap=Gap("log", 2.0, 1.5)),
             batch_size=n, batch=True)
    cap = (a.shape[1], b.shape[1])
    g = gpu_alg.m16.create_solver(*cap, gpu_alg.m16.create_options(o)).solve_indexed_for_alignment(a, b, table, ln)
    r = oracle_alg.m16.create_solver(*cap, oracle_alg.m16.create_options(o)).solve_indexed_for_alignment(
        a, b, table, ln)
    for k in range(n):
        assert g[k].score == r[k].score, (k, g[k].score, r[k].score)
        assert np.array_equal(np.asarray(g[k].s_to_t), np.asarray(r[k].s_to_t)), k
        assert np.array_equal(np.asarray(g[k].t_to_s), np.asarray(r[k].t_to_s)), k
