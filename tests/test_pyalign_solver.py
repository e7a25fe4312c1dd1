"""pyalign's own Python solver over this library's module interface (CPU only).

Where the reference's checkout is available (PYALIGN_REFERENCE = its root; skipped
otherwise), a bag of DNA problems shaped like the batched workload (half of them a query
and a mutated copy) is solved through ``pyalign.solve.LocalSolver(AffineGapCost(5, 2),
codomain=Alignment).solve(problems)`` -- Solver._solve_bag, ProblemBag.batches, the
indexed form's prepare and the native module's solve_indexed_for_alignment (solve.py:536-573,
instance.py:230-275, solve.py:399-432) -- with the oracle registered as the native module,
and then again with this library's opt-in replacements of the grouping
(prepare.patch_batches) and of the encoding (prepare.patch_prepare, host rows).  Scores and
alignment edges must be equal problem by problem.  It runs in a child process: importing
pyalign registers the native module for the whole interpreter.
"""

import os
import subprocess
import sys

import pytest

REF = os.environ.get("PYALIGN_REFERENCE")
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys, types, functools, importlib.machinery
import numpy as np
repo, ref = sys.argv[1], sys.argv[2]
sys.path[:0] = [repo, ref, repo + "/tests/golden"]
import make_golden
make_golden.install_shims()
import oracle.algorithm as oalg
make_golden.register_native(oalg)
import pyalign.problems, pyalign.solve, pyalign.gaps
from pyalign_gb300 import prepare
import bench

a, b, ls, lt, _ = bench.make_workload(300, 77, lo=20, hi=160)
letters = np.array(list("ACGT"))
pf = pyalign.problems.alphabetic("ACGT", pyalign.problems.Equality(eq=2, ne=-3))
problems = [pf.new_problem("".join(letters[a[k, :ls[k]]]), "".join(letters[b[k, :lt[k]]])) for k in range(len(ls))]

def run():
    solver = pyalign.solve.LocalSolver(gap_cost=pyalign.gaps.AffineGapCost(5, 2), codomain=pyalign.solve.Alignment)
    return [(r.score, r.edges.tolist()) for r in solver.solve(problems)]

ref_out = run()
prepare.patch_batches()
prepare.patch_prepare()
ours = run()
assert len(ours) == len(ref_out) == len(problems)
bad = [k for k in range(len(problems)) if ours[k] != ref_out[k]]
assert not bad, bad[:10]
assert any(r[0] > 0 for r in ours)
print("ok", len(problems))
'''


@pytest.mark.skipif(not REF, reason="PYALIGN_REFERENCE (the reference checkout) not set")
def test_pyalign_solver_with_bag_patches():
    r = subprocess.run([sys.executable, "-c", CHILD, REPO, REF], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok 300" in r.stdout
