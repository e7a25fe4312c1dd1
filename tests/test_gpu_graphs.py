"""Repeated device-resident solves and their CUDA graph (needs a GPU).

A solver that gets the same device-resident solve twice in a row (same lengths, buffers,
options) skips planning and staging and, from the second repetition on, launches the
device work as one CUDA graph.  The graph reads the inputs at launch, so new contents in
the same buffers must be seen; other lengths must re-plan.  Every result is compared with
the same solve on a solver that never caches (PA_GRAPHS=0), bit for bit.
"""

import ctypes
import types

import numpy as np
import pytest

from _cases import Gap

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from pyalign_gb300 import build
    build.build()
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device visible")
    from pyalign_gb300 import algorithm as alg
    from pyalign_gb300 import autograd as ag
    return torch, alg, ag


def _batch_solver(alg, torch, n, n_s, n_t):
    opts = {"solver": alg.Type.ALIGNMENT, "direction": alg.Direction.MAXIMIZE, "batch": True, "batch_size": n,
            "return_dup": False, "locality": alg.Locality.LOCAL,
            "codomain": types.SimpleNamespace(detail=alg.Detail.ALIGNMENT, count=alg.Count.ONE),
            "gap_cost": Gap("affine", 5.0, 2.0)}
    solver = alg.m16.create_solver(n_s, n_t, alg.m16.create_options(opts))
    alg.check(alg.lib().pa_solver_set_stream(solver.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return solver


def _timings(alg, solver):
    ms4 = (ctypes.c_float * 4)()
    nl = ctypes.c_int32(0)
    alg.check(alg.lib().pa_solver_last_timings(solver.handle, ms4, ctypes.byref(nl)))
    return list(ms4)


def _solve_batch(alg, torch, solver, a_d, b_d, t_d, ln, sc, mp):
    """pa_solve_batch with device codes/table and the device outputs sc, mp (reset first);
    returns (scores, maps)."""
    P = ctypes.POINTER
    n = a_d.shape[0]
    sizes = np.minimum(ln[0], ln[1]).astype(np.int64)
    offs = np.zeros(n, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    sc.fill_(float("nan"))
    mp.fill_(-7)
    length = np.ascontiguousarray(ln, dtype=np.int32)
    bt = alg.Batch(form=1, location=1, batch=n, n_s=a_d.shape[1], n_t=b_d.shape[1],
                   a=ctypes.cast(a_d.data_ptr(), P(ctypes.c_uint32)), b=ctypes.cast(b_d.data_ptr(), P(ctypes.c_uint32)),
                   table=ctypes.cast(t_d.data_ptr(), P(ctypes.c_float)), table_rows=4, table_cols=4,
                   length=length.ctypes.data_as(P(ctypes.c_int32)))
    alg.check(alg.lib().pa_solve_batch(solver.handle, ctypes.byref(bt), ctypes.c_void_p(sc.data_ptr()),
                                       ctypes.c_void_p(mp.data_ptr()), offs.ctypes.data_as(P(ctypes.c_int64))))
    torch.cuda.synchronize()
    m = int(sizes.sum())
    return sc.cpu().numpy(), mp[:m].cpu().numpy()


def test_repeated_batch_solves(env, monkeypatch):
    torch, alg, ag = env
    rng = np.random.default_rng(5)
    n, n_s, n_t = 512, 300, 320
    ln = np.stack([rng.integers(1, n_s + 1, n), rng.integers(1, n_t + 1, n)]).astype(np.int32)
    a = rng.integers(0, 4, size=(n, n_s)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, n_t)).astype(np.uint32)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    a_d = torch.from_numpy(a.view(np.int32)).cuda()
    b_d = torch.from_numpy(b.view(np.int32)).cuda()
    t_d = torch.from_numpy(table).cuda()
    sc = torch.empty(n, device="cuda")
    mp = torch.empty(int(np.minimum(ln[0], ln[1]).sum()), dtype=torch.int32, device="cuda")
    sc_r, mp_r = torch.empty_like(sc), torch.empty_like(mp)

    monkeypatch.setenv("PA_GRAPHS", "0")
    ref_solver = _batch_solver(alg, torch, n, n_s, n_t)
    want = _solve_batch(alg, torch, ref_solver, a_d, b_d, t_d, ln, sc_r, mp_r)
    monkeypatch.delenv("PA_GRAPHS")

    solver = _batch_solver(alg, torch, n, n_s, n_t)
    for rep in range(4):  # planned, cached plan + captured graph, graph, graph
        got = _solve_batch(alg, torch, solver, a_d, b_d, t_d, ln, sc, mp)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), rep
        ms = _timings(alg, solver)
        assert ms[1] > 0 and ms[2] > 0, (rep, ms)  # the phases are timed on replays too

    # new contents in the same buffers: the graph reads them at launch
    a_d.copy_(torch.from_numpy(rng.integers(0, 4, size=(n, n_s)).astype(np.int32)))
    got = _solve_batch(alg, torch, solver, a_d, b_d, t_d, ln, sc, mp)
    monkeypatch.setenv("PA_GRAPHS", "0")
    want2 = _solve_batch(alg, torch, ref_solver, a_d, b_d, t_d, ln, sc_r, mp_r)
    monkeypatch.delenv("PA_GRAPHS")
    assert np.array_equal(got[0], want2[0]) and np.array_equal(got[1], want2[1])
    assert not np.array_equal(want2[0], want[0])

    # other lengths: planned anew
    ln2 = ln.copy()
    ln2[0, :7] = 1
    got = _solve_batch(alg, torch, solver, a_d, b_d, t_d, ln2, sc, mp)
    monkeypatch.setenv("PA_GRAPHS", "0")
    want3 = _solve_batch(alg, torch, ref_solver, a_d, b_d, t_d, ln2, sc_r, mp_r)
    assert np.array_equal(got[0], want3[0]) and np.array_equal(got[1], want3[1])


@pytest.mark.parametrize("G", ["1", "8", "16"])
def test_repeated_block_kernel_solves(env, monkeypatch, G):
    """Repeats and graph replays of a plan on the 4 x 4 block kernel keep that kernel (and its
    traceback layout) on every repetition, with the results of an uncached solve."""
    torch, alg, ag = env
    monkeypatch.setenv("PA_DP_BLOCK", "1")
    monkeypatch.setenv("PA_GROUP_WIDTH", G)
    rng = np.random.default_rng(50 + int(G))
    n, n_s, n_t = 301, 260, 270
    ln = np.stack([rng.integers(1, n_s + 1, n), rng.integers(1, n_t + 1, n)]).astype(np.int32)
    a = rng.integers(0, 4, size=(n, n_s)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, n_t)).astype(np.uint32)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    a_d = torch.from_numpy(a.view(np.int32)).cuda()
    b_d = torch.from_numpy(b.view(np.int32)).cuda()
    t_d = torch.from_numpy(table).cuda()
    sc = torch.empty(n, device="cuda")
    mp = torch.empty(int(np.minimum(ln[0], ln[1]).sum()), dtype=torch.int32, device="cuda")
    sc_r, mp_r = torch.empty_like(sc), torch.empty_like(mp)
    monkeypatch.setenv("PA_GRAPHS", "0")
    ref_solver = _batch_solver(alg, torch, n, n_s, n_t)
    want = _solve_batch(alg, torch, ref_solver, a_d, b_d, t_d, ln, sc_r, mp_r)
    assert ref_solver.last_plan()["kernel"] == "16-bit twins, 4x4 blocks", ref_solver.last_plan()
    monkeypatch.delenv("PA_GRAPHS")
    solver = _batch_solver(alg, torch, n, n_s, n_t)
    for rep in range(4):  # planned, cached plan + captured graph, graph, graph
        got = _solve_batch(alg, torch, solver, a_d, b_d, t_d, ln, sc, mp)
        plan = solver.last_plan()
        assert plan["kernel"] == "16-bit twins, 4x4 blocks" and plan["G"] == int(G), (rep, plan)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), rep


@pytest.mark.parametrize("widths", ["8,16,16,32", "1,4,32,2"])
def test_repeated_bucket_width_solves(env, monkeypatch, widths):
    """Repeats and graph replays of a plan with a group width per length bucket of |s| keep
    the widths (the segments of the launch, each pair's traceback layout) on every
    repetition, with the results of an uncached one-width solve."""
    torch, alg, ag = env
    rng = np.random.default_rng(sum(map(int, widths.split(","))))
    n, n_s, n_t = 301, 700, 300
    ln = np.stack([rng.integers(1, n_s + 1, n), rng.integers(1, n_t + 1, n)]).astype(np.int32)
    a = rng.integers(0, 4, size=(n, n_s)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, n_t)).astype(np.uint32)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    a_d = torch.from_numpy(a.view(np.int32)).cuda()
    b_d = torch.from_numpy(b.view(np.int32)).cuda()
    t_d = torch.from_numpy(table).cuda()
    sc = torch.empty(n, device="cuda")
    mp = torch.empty(int(np.minimum(ln[0], ln[1]).sum()), dtype=torch.int32, device="cuda")
    sc_r, mp_r = torch.empty_like(sc), torch.empty_like(mp)
    monkeypatch.setenv("PA_GRAPHS", "0")
    monkeypatch.setenv("PA_TUNE", "0")
    monkeypatch.setenv("PA_DP_MODE", "groups")
    ref_solver = _batch_solver(alg, torch, n, n_s, n_t)
    want = _solve_batch(alg, torch, ref_solver, a_d, b_d, t_d, ln, sc_r, mp_r)
    assert ref_solver.last_plan()["bucket_widths"] is None, ref_solver.last_plan()
    monkeypatch.delenv("PA_GRAPHS")
    monkeypatch.setenv("PA_BUCKET_WIDTHS", widths)
    solver = _batch_solver(alg, torch, n, n_s, n_t)
    for rep in range(4):  # planned, cached plan + captured graph, graph, graph
        got = _solve_batch(alg, torch, solver, a_d, b_d, t_d, ln, sc, mp)
        plan = solver.last_plan()
        assert plan["kernel"] == "16-bit twins, two-column", (rep, plan)
        assert plan["bucket_widths"] == [int(g) for g in widths.split(",")], (rep, plan)
        assert plan["graph"] == (rep >= 1), (rep, plan)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), rep


def test_repeated_dense_paths_and_gradients(env, monkeypatch):
    """The autograd front end (pa_solve_dense_paths): repeated forward + backward on one
    similarity buffer whose contents change in place."""
    torch, alg, ag = env
    g = torch.Generator(device="cuda").manual_seed(3)
    B, ns, nt = 96, 200, 170
    rng = np.random.default_rng(9)
    lengths = np.stack([rng.integers(1, ns + 1, B), rng.integers(1, nt + 1, B)], axis=1)
    S = torch.randn(B, ns, nt, device="cuda", generator=g)

    def run():
        return ag.alignment_score(S, lengths, 0.5, 0.1, "global").clone()

    monkeypatch.setenv("PA_GRAPHS", "0")
    want = run()
    monkeypatch.delenv("PA_GRAPHS")
    for rep in range(4):
        assert torch.equal(run(), want), rep
    S.mul_(-1.0).add_(0.25)
    got = run()
    monkeypatch.setenv("PA_GRAPHS", "0")
    assert torch.equal(got, run())
    assert not torch.equal(got, want)


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("chunks,widths", [(None, None), ("3", None), ("3", "4,8,32,16"), ("5", "2,16,8,32")])
def test_repeated_host_batch_solves(env, monkeypatch, chunks, widths, pinned):
    """pa_solve_batch with host buffers: a repeat reuses the plan and staged metadata (no
    graph) -- with PA_CHUNKS=3 as a pipeline of three pair ranges whose uploads, DPs, walks and
    map downloads overlap, also with a group width per length bucket (segments per chunk);
    new contents and new lengths are solved exactly as by a one-width solver that never
    caches; maps in pageable or pinned host memory."""
    torch, alg, ag = env
    if chunks:
        monkeypatch.setenv("PA_CHUNKS", chunks)
    P = ctypes.POINTER
    rng = np.random.default_rng(17)
    n, n_s, n_t = 700, 260, 300
    ln = np.stack([rng.integers(0, n_s + 1, n), rng.integers(1, n_t + 1, n)]).astype(np.int32)
    a = rng.integers(0, 4, size=(n, n_s)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, n_t)).astype(np.uint32)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)

    def solve(solver, a, b, ln, pin=False):
        sizes = np.minimum(ln[0], ln[1]).astype(np.int64)
        offs = np.zeros(n, np.int64)
        offs[1:] = np.cumsum(sizes)[:-1]
        sc = np.full(n, np.nan, np.float32)
        if pin:
            mp = torch.full((max(1, int(sizes.sum())),), -7, dtype=torch.int32).pin_memory().numpy()
        else:
            mp = np.full(max(1, int(sizes.sum())), -7, np.int32)
        length = np.ascontiguousarray(ln, dtype=np.int32)
        bt = alg.Batch(form=1, location=0, batch=n, n_s=n_s, n_t=n_t,
                       a=a.ctypes.data_as(P(ctypes.c_uint32)), b=b.ctypes.data_as(P(ctypes.c_uint32)),
                       table=table.ctypes.data_as(P(ctypes.c_float)), table_rows=4, table_cols=4,
                       length=length.ctypes.data_as(P(ctypes.c_int32)))
        alg.check(alg.lib().pa_solve_batch(solver.handle, ctypes.byref(bt), sc.ctypes.data_as(ctypes.c_void_p),
                                           mp.ctypes.data_as(ctypes.c_void_p), offs.ctypes.data_as(P(ctypes.c_int64))))
        return sc, mp

    def ref_solve(a, b, ln):
        with monkeypatch.context() as m:
            m.setenv("PA_GRAPHS", "0")
            if widths:
                m.delenv("PA_BUCKET_WIDTHS")
                m.setenv("PA_TUNE", "0")
            return solve(ref, a, b, ln)

    if widths:
        monkeypatch.setenv("PA_BUCKET_WIDTHS", widths)
        monkeypatch.setenv("PA_DP_MODE", "groups")
    ref = _batch_solver(alg, torch, n, n_s, n_t)
    want = ref_solve(a, b, ln)
    solver = _batch_solver(alg, torch, n, n_s, n_t)
    for rep in range(3):
        got = solve(solver, a, b, ln, pinned)
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), rep
        assert not solver.last_plan()["graph"]
        if widths:
            assert solver.last_plan()["bucket_widths"] == [int(g) for g in widths.split(",")], solver.last_plan()
    a[:, :] = rng.integers(0, 4, size=(n, n_s))              # new contents, same host buffer
    got = solve(solver, a, b, ln, pinned)
    want2 = ref_solve(a, b, ln)
    assert np.array_equal(got[0], want2[0]) and np.array_equal(got[1], want2[1])
    ln2 = ln.copy()
    ln2[1, :11] = 3                                           # new lengths: planned anew
    got = solve(solver, a, b, ln2, pinned)
    want3 = ref_solve(a, b, ln2)
    assert np.array_equal(got[0], want3[0]) and np.array_equal(got[1], want3[1])


def test_host_maps_need_packed_offsets(env):
    """Host maps are staged at the packed offsets: other offsets are refused before any work."""
    torch, alg, ag = env
    P = ctypes.POINTER
    n, n_s, n_t = 8, 20, 20
    rng = np.random.default_rng(3)
    a = rng.integers(0, 4, size=(n, n_s)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, n_t)).astype(np.uint32)
    table = np.eye(4, dtype=np.float32)
    length = np.full((2, n), 20, np.int32)
    offs = np.arange(n, dtype=np.int64) * 25                 # gaps between the maps
    sc = np.zeros(n, np.float32)
    mp = np.zeros(n * 25, np.int32)
    bt = alg.Batch(form=1, location=0, batch=n, n_s=n_s, n_t=n_t,
                   a=a.ctypes.data_as(P(ctypes.c_uint32)), b=b.ctypes.data_as(P(ctypes.c_uint32)),
                   table=table.ctypes.data_as(P(ctypes.c_float)), table_rows=4, table_cols=4,
                   length=length.ctypes.data_as(P(ctypes.c_int32)))
    solver = _batch_solver(alg, torch, n, n_s, n_t)
    with pytest.raises(ValueError, match="prefix sums"):
        alg.check(alg.lib().pa_solve_batch(solver.handle, ctypes.byref(bt), sc.ctypes.data_as(ctypes.c_void_p),
                                           mp.ctypes.data_as(ctypes.c_void_p), offs.ctypes.data_as(P(ctypes.c_int64))))


def test_direct_maps_result_refuses_map_reads(env):
    """pa_solve_batch_result writes the maps into the caller's array; the result object it
    returns has the scores and refuses to hand out maps it does not hold."""
    torch, alg, ag = env
    P = ctypes.POINTER
    rng = np.random.default_rng(8)
    n, n_s, n_t = 40, 50, 60
    ln = np.stack([rng.integers(0, n_s + 1, n), rng.integers(1, n_t + 1, n)]).astype(np.int32)
    a = rng.integers(0, 4, size=(n, n_s)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, n_t)).astype(np.uint32)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    sizes = np.minimum(ln[0], ln[1]).astype(np.int64)
    offs = np.zeros(n, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    maps = np.full(int(sizes.sum()), -7, np.int32)
    bt = alg.Batch(form=1, location=0, batch=n, n_s=n_s, n_t=n_t, a=a.ctypes.data_as(P(ctypes.c_uint32)),
                   b=b.ctypes.data_as(P(ctypes.c_uint32)), table=table.ctypes.data_as(P(ctypes.c_float)),
                   table_rows=4, table_cols=4, length=ln.ctypes.data_as(P(ctypes.c_int32)))
    solver = _batch_solver(alg, torch, n, n_s, n_t)
    h = alg._P()
    alg.check(alg.lib().pa_solve_batch_result(solver.handle, ctypes.byref(bt), alg._ip(maps),
                                              offs.ctypes.data_as(alg._PL), ctypes.byref(h)))
    res = alg._Result(h)
    sc = np.zeros(n, np.float32)
    alg.check(alg.lib().pa_result_export(res.ptr, alg._fp(sc), None, None))
    m0 = np.zeros(max(1, int(sizes[0])), np.int32)
    assert alg.lib().pa_result_alignment(res.ptr, 0, alg._ip(m0)) != 0
    # the same bag through pa_solve_batch: equal scores and maps
    sc2 = np.zeros(n, np.float32)
    maps2 = np.full_like(maps, -9)
    alg.check(alg.lib().pa_solve_batch(solver.handle, ctypes.byref(bt), sc2.ctypes.data_as(ctypes.c_void_p),
                                       maps2.ctypes.data_as(ctypes.c_void_p), offs.ctypes.data_as(alg._PL)))
    assert np.array_equal(maps, maps2)
    has = np.array([alg.lib().pa_result_has_alignment(res.ptr, k) for k in range(n)], bool)
    assert np.array_equal(sc[has], sc2[has])


def test_pipelined_python_api_repeats(env, monkeypatch, oracle_alg):
    """The native module's solve_indexed_for_alignment repeated with host arrays, pipelined in
    four chunks (maps straight into the results' array), against the oracle."""
    torch, alg, ag = env
    from _cases import compare, options
    monkeypatch.setenv("PA_CHUNKS", "4")
    rng = np.random.default_rng(23)
    n = 301
    ls = rng.integers(0, 200, size=n)
    lt = rng.integers(1, 220, size=n)
    a = rng.integers(0, 4, size=(n, 200)).astype(np.uint32)
    b = rng.integers(0, 4, size=(n, 220)).astype(np.uint32)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    ln = np.stack([ls, lt]).astype(np.uint16)
    opts = dict(options(alg, locality="local", detail="alignment", gap=Gap("affine", 5.0, 2.0)), batch_size=n)
    solver = alg.m16.create_solver(200, 220, alg.m16.create_options(opts))
    oracle = oracle_alg.m16.create_solver(200, 220, oracle_alg.m16.create_options(opts))
    want = oracle.solve_indexed_for_alignment(a, b, table, ln)
    for rep in range(3):
        got = solver.solve_indexed_for_alignment(a, b, table, ln)
        d = compare("alignment", got, want, n)
        assert d is None, (rep, d)
