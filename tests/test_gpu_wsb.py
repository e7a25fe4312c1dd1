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
