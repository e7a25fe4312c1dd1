"""The allocation-free score entry point against the regular one (needs a GPU).

pa_solve_indexed_for_score_noalloc serves callers that cannot allocate device memory
while they run (a process that owns its HBM through a preallocated pool, or code where a
cudaMalloc would stall or fail mid-request): the caller passes device inputs and outputs,
and the entry point keeps its scratch in one static device array.  These tests call it
through the C ABI twice in a row -- with different shapes, gap costs and directions, so
stale scratch from the first call would show -- and require the same scores as
pa_solve_indexed_for_score, bit for bit, as every parity test here does.
"""

import ctypes
import types

import numpy as np
import pytest

from _cases import Gap, pack, random_pairs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0 or not torch.cuda.is_available():
        pytest.fail("no CUDA device visible")
    L = alg.lib()
    vp, i64 = ctypes.c_void_p, ctypes.c_int64
    L.pa_solve_indexed_for_score_noalloc.restype = ctypes.c_int32
    L.pa_solve_indexed_for_score_noalloc.argtypes = [vp, vp, vp, i64, i64, i64, vp, i64, i64, vp, vp, vp, vp]
    return torch, alg, L


def _options_dict(alg, locality, direction, gap, batch):
    return {
        "solver": alg.Type.ALIGNMENT, "direction": alg.Direction.__members__[direction.upper()],
        "batch": True, "batch_size": batch, "return_dup": False,
        "locality": alg.Locality.__members__[locality.upper()],
        "codomain": types.SimpleNamespace(detail=alg.Detail.SCORE, count=alg.Count.ONE),
        "gap_cost": gap,
    }


def _c_options(alg, locality, direction, gap):
    o = alg._Options()
    o.type = 0
    o.direction = int(alg.Direction.__members__[direction.upper()])
    o.locality = int(alg.Locality.__members__[locality.upper()])
    o.detail, o.count = 0, 0
    sc = gap.to_special_case()
    if "affine" in sc:
        u, v = sc["affine"]
        o.gap_kind = 1
        o.affine_u_s = o.affine_u_t = float(np.float32(v))   # Gotoh u = extend
        o.affine_v_s = o.affine_v_t = float(np.float32(u))   # Gotoh v = open - extend
    else:
        o.gap_kind = 0
        o.linear_s = o.linear_t = float(np.float32(sc["linear"]))
    return o


def _both(env, pairs, table, locality, direction, gap):
    torch, alg, L = env
    n = len(pairs)
    a, b, ln = pack(pairs, n)
    mod = alg.m16
    solver = mod.create_solver(a.shape[1], b.shape[1], mod.create_options(
        _options_dict(alg, locality, direction, gap, n)))
    want = solver.solve_indexed_for_score(a, b, table, ln)

    dev = "cuda"
    a_d = torch.from_numpy(a.view(np.int32)).to(dev)
    b_d = torch.from_numpy(b.view(np.int32)).to(dev)
    t_d = torch.from_numpy(table).to(dev)
    ls_d = torch.from_numpy(ln[0].astype(np.int32)).to(dev)
    lt_d = torch.from_numpy(ln[1].astype(np.int32)).to(dev)
    out = torch.full((n,), float("nan"), dtype=torch.float32, device=dev)
    o = _c_options(alg, locality, direction, gap)
    stream = torch.cuda.current_stream().cuda_stream
    st = L.pa_solve_indexed_for_score_noalloc(
        ctypes.addressof(o), a_d.data_ptr(), b_d.data_ptr(), n, a.shape[1], b.shape[1], t_d.data_ptr(),
        table.shape[0], table.shape[1], ls_d.data_ptr(), lt_d.data_ptr(), out.data_ptr(), stream)
    alg.check(st)
    torch.cuda.synchronize()
    return want, out.cpu().numpy()


def test_noalloc_matches_regular_entry_two_calls(env):
    rng = np.random.default_rng(2024)
    dna = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(dna, 2.0)
    pairs1 = random_pairs(rng, 300, 50, 400, alphabet=4, related=0.6)
    want1, got1 = _both(env, pairs1, dna, "local", "maximize", Gap("affine", 5.0, 2.0))
    assert np.array_equal(want1, got1), np.nonzero(want1 != got1)[0][:10]

    ftab = rng.normal(size=(6, 6)).astype(np.float32)
    ftab = ((ftab + ftab.T) / 2).astype(np.float32)
    pairs2 = random_pairs(rng, 120, 0, 700, alphabet=6, related=0.4)
    want2, got2 = _both(env, pairs2, ftab, "global", "minimize", Gap("linear", 1.5))
    assert np.array_equal(want2, got2), np.nonzero(want2 != got2)[0][:10]

    want3, got3 = _both(env, pairs1[:64], dna, "semiglobal", "maximize", Gap("affine", 10.0, 1.0))
    assert np.array_equal(want3, got3)


def test_noalloc_global_affine_fractional_costs(env, oracle_alg):
    """Global affine borders with fractional costs (open 2.7, extend 0.3) and a capacity with
    n_s != n_t: the border vector the entry point builds on the device must equal the
    regular entry's and the oracle's, bit for bit, on two calls in a row."""
    rng = np.random.default_rng(2025)
    ftab = rng.normal(size=(5, 5)).astype(np.float32)
    for k, direction in enumerate(("maximize", "minimize")):
        hi = 300 + 200 * k
        pairs = random_pairs(rng, 90 + 40 * k, 0, hi, alphabet=5, related=0.5)
        pairs.append((rng.integers(0, 5, size=7).astype(np.uint32), rng.integers(0, 5, size=hi + 41).astype(np.uint32)))
        gap = Gap("affine", 2.7, 0.3)
        want, got = _both(env, pairs, ftab, "global", direction, gap)
        assert np.array_equal(want, got), np.nonzero(want != got)[0][:10]
        n = len(pairs)
        a, b, ln = pack(pairs, n)
        assert a.shape[1] != b.shape[1]
        osol = oracle_alg.m16.create_solver(a.shape[1], b.shape[1], oracle_alg.m16.create_options(
            _options_dict(oracle_alg, "global", direction, gap, n)))
        ref = np.asarray(osol.solve_indexed_for_score(a, b, ftab, ln))
        assert np.array_equal(ref, got), np.nonzero(ref != got)[0][:10]


def test_noalloc_rejects_sizes_beyond_maximum(env):
    torch, alg, L = env
    o = _c_options(alg, "local", "maximize", Gap("linear", 1.0))
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = dummy.data_ptr()
    st = L.pa_solve_indexed_for_score_noalloc(ctypes.addressof(o), p, p, 65537, 4, 4, p, 2, 2, p, p, p, None)
    assert st == 2 and b"PA_NOALLOC_MAX_BATCH" in L.pa_last_error()
    st = L.pa_solve_indexed_for_score_noalloc(ctypes.addressof(o), p, p, 4, 5000, 4, p, 2, 2, p, p, p, None)
    assert st == 2 and b"PA_NOALLOC_MAX_LEN" in L.pa_last_error()
