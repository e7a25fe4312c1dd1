"""The oracle against the reference's own known-answer tests (CPU only).

Each recorded native call from pyalign/tests/*.py is replayed on the oracle, and the
scores and edge sets that the reference test asserted are checked exactly as
pyalign/test.py:24-34 does (score to `places` decimals, sorted edge lists equal).
"""

import pytest

from _replay import drain, edges_of, load_golden, run_call

GOLDEN = load_golden()


def _check(results, expected):
    for x in results:
        assert round(abs(x.score - expected["score"]), expected["places"]) == 0
    got = sorted(edges_of(x) for x in results)
    want = sorted(expected["edges"])
    assert got == want


@pytest.mark.parametrize("check", GOLDEN["checks"], ids=lambda c: f'{c["test"].split(".")[-1]}-call{c["call"]}-lane{c["lane"]}')
def test_oracle_matches_reference_test(oracle_alg, check):
    call = GOLDEN["calls"][check["call"]]
    _, res, _ = run_call(oracle_alg, call)
    item = res[check["lane"]]
    if call["method"].endswith("alignment_iterator"):
        results = drain(item)
    else:
        results = [item]
    _check(results, check)


def test_all_reference_tests_recorded():
    assert GOLDEN["tests_run"] == 9
    names = {c["test"].split(".")[-1] for c in GOLDEN["checks"]}
    assert {"test_simd", "test_CC_ACCT", "test_aatcg_aacg", "test_cg_ccga"} <= names
