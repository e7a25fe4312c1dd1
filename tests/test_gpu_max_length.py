"""Pairs at the index types' length limits (needs a GPU).

The reference's MatrixFactory refuses lengths past half the index type's range
(solver.h:487-503): 16,383 for m16.  A pair of 16,383 x 16,383 (268 M cells) with m16 and
one of 20,000 x 18,000 with m32 are solved on the GPU; their scores equal the oracle's
memory-lean score bit for bit, and each returned alignment is a valid local / semiglobal
alignment whose re-evaluated score (matches along the map, affine gap costs between
consecutive aligned pairs) is the returned score.  The oracle's full alignment matrices
would need ~10 GB per pair at these sizes, hence the re-evaluation.
"""

import numpy as np
import pytest

from _cases import Gap, options

pytestmark = pytest.mark.gpu

OPEN, EXT = 5.0, 2.0


@pytest.fixture(scope="module")
def gpu_alg():
    from pyalign_gb300 import build
    build.build()
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() == 0:
        pytest.fail("no CUDA device visible")
    return alg


def _rescore(a, b, table, mp, ls, lt):
    """Score of the alignment a map describes (s_to_t when |s| <= |t|, else t_to_s)."""
    if ls <= lt:
        pairs = [(i, int(j)) for i, j in enumerate(mp) if j >= 0]
    else:
        pairs = sorted((int(i), j) for j, i in enumerate(mp) if i >= 0)
    if not pairs:
        return None
    ii = np.array([p[0] for p in pairs])
    jj = np.array([p[1] for p in pairs])
    assert np.all(np.diff(ii) > 0) and np.all(np.diff(jj) > 0), "the map is not an alignment"
    score = float(table[a[ii], b[jj]].astype(np.float64).sum())

    def w(k):  # pyalign's AffineGapCost(open, extend): extend * k + (open - extend)
        return EXT * k + (OPEN - EXT) if k > 0 else 0.0

    di, dj = np.diff(ii) - 1, np.diff(jj) - 1
    score -= sum(w(int(k)) for k in di) + sum(w(int(k)) for k in dj)
    return score  # local and semiglobal: the ends cost nothing


@pytest.mark.parametrize("bits,ls,lt,locality", [(16, 16383, 16383, "local"), (16, 16383, 1, "local"),
                                                 (32, 20000, 18000, "semiglobal")])
def test_pairs_at_the_length_limit(gpu_alg, oracle_alg, bits, ls, lt, locality):
    rng = np.random.default_rng(ls + lt + bits)
    a = rng.integers(0, 4, size=(1, ls)).astype(np.uint32)
    b = rng.integers(0, 4, size=(1, lt)).astype(np.uint32)
    # a related stretch, so the optimum is a long alignment with gaps
    k = min(ls, lt) // 2
    b[0, :k] = a[0, :k]
    mut = rng.random(k) < 0.1
    b[0, :k][mut] = rng.integers(0, 4, int(mut.sum()))
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    ln = np.array([[ls], [lt]], np.uint16)  # pyalign passes uint16 lengths (solve.py:350, 409)
    o = dict(options(gpu_alg, locality=locality, detail="alignment", gap=Gap("affine", OPEN, EXT)), batch_size=1)
    mod = gpu_alg.m16 if bits == 16 else gpu_alg.m32
    solver = mod.create_solver(ls, lt, mod.create_options(o))
    res = solver.solve_indexed_for_alignment(a, b, table, ln)
    omod = oracle_alg.m16 if bits == 16 else oracle_alg.m32
    osol = omod.create_solver(ls, lt, omod.create_options(o))
    osc, _ = oracle_alg.batch_scores_lean(osol, a, b, table, np.array([ls]), np.array([lt]))
    assert res[0].score == osc[0], (res[0].score, osc[0])
    mp = np.asarray(res[0].s_to_t if ls <= lt else res[0].t_to_s)
    got = _rescore(a[0], b[0], table, mp, ls, lt)
    assert got is not None and got == float(osc[0]), (got, osc[0])
