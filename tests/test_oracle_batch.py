"""The oracle's threaded batch helpers against its one-pair solver (CPU only).

Parity checks at full workload sizes use three batch forms of the oracle: scores and
alignment maps on host threads (batch_alignments), a two-rows-per-layer score for pairs of
5000 x 10000 cells (batch_scores_lean), and the FP64 twin over float32 matrices
(batch_f64).  Each must give what the oracle's own per-pair solver gives -- the solver that
the reference's unit tests pin -- bit for bit.
"""

import numpy as np
import pytest

from _cases import Gap, options


@pytest.mark.parametrize("locality", ["local", "global", "semiglobal"])
@pytest.mark.parametrize("direction", ["maximize", "minimize"])
def test_lean_score_and_batch_alignments_equal_per_pair_solver(oracle_alg, locality, direction):
    rng = np.random.default_rng(hash((locality, direction)) % 2**31)
    for gap in (Gap("linear", 2.0), Gap("affine", 5.0, 2.0), Gap("affine", 2.7, 0.3)):
        n, w = 120, 48
        ls = rng.integers(0, w + 1, n)
        lt = rng.integers(0, w + 1, n)
        a = rng.integers(0, 5, (n, w)).astype(np.uint32)
        b = rng.integers(0, 5, (n, w)).astype(np.uint32)
        table = (rng.integers(-4, 6, (5, 5)) * 1.5).astype(np.float32)
        ln = np.stack([ls, lt]).astype(np.uint16)
        for detail in ("score", "alignment"):
            o = dict(options(oracle_alg, locality=locality, direction=direction, detail=detail, gap=gap),
                     batch_size=n, batch=True)
            s = oracle_alg.m16.create_solver(w, w, oracle_alg.m16.create_options(o))
            if detail == "score":
                ref = np.asarray(s.solve_indexed_for_score(a, b, table, ln))
                lean, _ = oracle_alg.batch_scores_lean(s, a, b, table, ls, lt, threads=3)
                assert np.array_equal(ref, lean), (gap, np.nonzero(ref != lean))
            else:
                res = s.solve_indexed_for_alignment(a, b, table, ln)
                sc, mp, offs, _ = oracle_alg.batch_alignments(s, a, b, table, ls, lt, threads=3)
                for k in range(n):
                    m = res[k].s_to_t if ls[k] <= lt[k] else res[k].t_to_s
                    assert res[k].score == sc[k] or (np.isinf(res[k].score) and np.isinf(sc[k])), (gap, k)
                    assert np.array_equal(np.asarray(m), mp[offs[k]:offs[k + 1]]), (gap, k)


def test_batch_f64_equals_float32_on_integer_matrices(oracle_alg):
    """On integer-valued matrices every value is exact in both precisions: the FP64 twin's
    scores equal the float32 solver's, and the term magnitude is at least |score|."""
    rng = np.random.default_rng(64)
    B, w = 40, 60
    ls = rng.integers(1, w + 1, B)
    lt = rng.integers(1, w + 1, B)
    S = rng.integers(-3, 4, (B, w, w)).astype(np.float32)
    for dtw, direction in ((False, "maximize"), (True, "minimize")):
        sc64, scale = oracle_alg.batch_f64(np.abs(S) if dtw else S, ls, lt, dtw=dtw, direction=direction,
                                           open_=3.0, extend=1.0, threads=2)
        o = dict(options(oracle_alg, dtw=dtw, locality="global", direction=direction, detail="score",
                         gap=None if dtw else Gap("affine", 3.0, 1.0)), batch_size=B, batch=True)
        s = oracle_alg.m16.create_solver(w, w, oracle_alg.m16.create_options(o))
        sim = np.ascontiguousarray((np.abs(S) if dtw else S).transpose(1, 2, 0))
        ref = np.asarray(s.solve_for_score(sim, np.stack([ls, lt]).astype(np.uint16)))
        assert np.array_equal(sc64, ref.astype(np.float64)), (dtw, sc64[:4], ref[:4])
        assert np.all(scale >= np.abs(sc64) - 1e-9)
