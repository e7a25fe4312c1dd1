"""Pin the oracle to the reference's own known-answer tests and record them as fixtures.

Run in the build container (where the reference checkout exists):

    python tests/golden/make_golden.py --reference <path of the pyalign checkout>

(or with PYALIGN_REFERENCE set to that path)

What it does:
1. Imports the reference's *Python* package (pyalign 0.4.4) from the checkout, with two
   missing pure-Python dependencies shimmed (``cached_property`` -> functools, and
   ``pymorton.interleave2``), and registers ``oracle/algorithm.py`` as the native module
   ``pyalign.algorithm.native.algorithm`` that pyalign/cpu.py:21-47 looks for.
2. Runs the reference's unittest suite (pyalign/tests/*.py).  Every assertion in it checks
   the oracle against the reference's golden vectors; the script fails if any test fails.
3. Records every native ``solve_*`` call made during those tests (the arrays crossing the
   Python/C++ boundary, the solver options) together with the expected scores and edge
   sets that the reference test asserted, into ``tests/golden/reference_tests.json``.

The GPU parity tests replay those calls through the C-ABI and compare with the expected
values; nothing at test time reads the reference checkout.
"""

import argparse
import functools
import importlib.machinery
import json
import warnings
import os
import sys
import types
import unittest

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _part1by1(n):
    n &= 0x0000ffff
    n = (n | (n << 8)) & 0x00FF00FF
    n = (n | (n << 4)) & 0x0F0F0F0F
    n = (n | (n << 2)) & 0x33333333
    n = (n | (n << 1)) & 0x55555555
    return n


def install_shims():
    cp = types.ModuleType("cached_property")
    cp.cached_property = functools.cached_property
    sys.modules.setdefault("cached_property", cp)
    pm = types.ModuleType("pymorton")
    pm.interleave2 = lambda x, y: _part1by1(int(x)) | (_part1by1(int(y)) << 1)
    sys.modules.setdefault("pymorton", pm)


def register_native(module):
    """Make pyalign.cpu.import_algorithm() return `module` (cpu.py:33-40)."""
    pkg = types.ModuleType("pyalign.algorithm.native")
    pkg.__path__ = []
    pkg.__spec__ = importlib.machinery.ModuleSpec("pyalign.algorithm.native", None, is_package=True)
    module.__spec__ = importlib.machinery.ModuleSpec("pyalign.algorithm.native.algorithm", None)
    pkg.algorithm = module
    sys.modules["pyalign.algorithm.native"] = pkg
    sys.modules["pyalign.algorithm.native.algorithm"] = module


def _gap_record(spec, cap):
    kind, val = spec
    if kind == "linear":
        return {"kind": "linear", "w": float(val)}
    if kind == "affine":
        # Gotoh (u, v) as the native side sees them: w(k) = u k + v
        return {"kind": "affine", "u": float(val[0]), "v": float(val[1])}
    return {"kind": "general", "costs": np.asarray(val.costs(cap + 1), dtype=np.float32).tolist()}


class Recorder:
    """Wraps oracle.algorithm and logs the native calls and their results."""

    def __init__(self, oracle_alg):
        self.alg = oracle_alg
        self.calls = []
        self.checks = []
        rec = self
        base = oracle_alg.Solver

        methods = [m for m in dir(base) if m.startswith("solve_")]

        class RecSolver(base):
            pass

        def make(name):
            orig = getattr(base, name)

            def wrapped(self, *args):
                call_id = len(rec.calls)
                entry = {"id": call_id, "method": name}
                o = self._opts
                entry["index_bits"] = o.index_bits
                entry["cap"] = [self._cap_s, self._cap_t]
                entry["options"] = {
                    "type": int(o.type), "direction": int(o.direction), "detail": int(o.detail),
                    "count": int(o.count), "locality": int(o.locality),
                    "return_dup": not o.remove_dup, "batch": bool(o.batch),
                    "gap_s": _gap_record(o.gap_s, self._cap_s),
                    "gap_t": _gap_record(o.gap_t, self._cap_t),
                }
                names = {"solve_for": ["sim", "len"], "solve_indexed_for": ["a", "b", "sim", "len"],
                         "solve_binary_for": ["a", "b", "eq", "ne", "len"]}
                key = name.split("_for_")[0] + "_for"
                entry["args"] = {k: (np.asarray(v).tolist() if not np.isscalar(v) else float(v))
                                 for k, v in zip(names[key], args)}
                # drain a second, independent result for the record
                shadow = orig(self, *args)
                entry["result"] = rec.describe(name, shadow)
                rec.calls.append(entry)
                out = orig(self, *args)
                if isinstance(out, tuple):
                    for lane, x in enumerate(out):
                        x._golden = (call_id, lane)
                return out

            return wrapped

        for m in methods:
            setattr(RecSolver, m, make(m))

        # tag alignments produced by iterators with their call/lane
        it_next = oracle_alg.AlignmentIterator.next

        def next_tagged(it):
            a = it_next(it)
            if a is not None and hasattr(it, "_golden"):
                a._golden = it._golden
            return a

        oracle_alg.AlignmentIterator.next = next_tagged

        for mod in (oracle_alg.m16, oracle_alg.m32):
            mod.Solver = RecSolver
            mod.create_solver = (lambda s, t, o, _S=RecSolver: _S(s, t, o))

    @staticmethod
    def describe(name, out):
        if name.endswith("for_score"):
            return {"scores": np.asarray(out, dtype=np.float64).tolist()}
        lanes = []
        for x in out:
            if name.endswith("alignment_iterator"):
                items = []
                while True:
                    a = x.next()
                    if a is None:
                        break
                    items.append({"score": a.score, "s_to_t": a.s_to_t.tolist()})
                lanes.append(items)
            elif name.endswith("for_alignment"):
                lanes.append({"score": x.score, "s_to_t": x.s_to_t.tolist()})
            else:
                lanes.append(None)  # solutions are compared live against the oracle
        return {"lanes": lanes}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PYALIGN_REFERENCE"),
                    required=not os.environ.get("PYALIGN_REFERENCE"),
                    help="root of the pyalign 0.4.4 checkout (default: $PYALIGN_REFERENCE)")
    ap.add_argument("--out", default=os.path.join(HERE, "reference_tests.json"))
    args = ap.parse_args()

    warnings.simplefilter("ignore", SyntaxWarning)
    sys.path.insert(0, REPO)
    sys.path.insert(0, args.reference)
    install_shims()
    import oracle.algorithm as oracle_alg
    oracle_alg.build()
    rec = Recorder(oracle_alg)
    register_native(oracle_alg)

    import pyalign  # noqa: F401  (the reference package)
    import pyalign.test

    orig_check = pyalign.test.TestCase._check_alignments

    def check(self, alignments, score, *edges, places=7):
        items = list(alignments)
        tags = {getattr(x._alignment, "_golden", None) for x in items}
        tags.discard(None)
        if len(tags) != 1:
            raise AssertionError(f"cannot attribute checked alignments to one native call: {tags}")
        call_id, lane = tags.pop()
        rec.checks.append({
            "test": self.id(), "call": call_id, "lane": lane, "score": float(score),
            "places": places, "edges": [list(map(list, e)) for e in edges]})
        return orig_check(self, items, score, *edges, places=places)

    pyalign.test.TestCase._check_alignments = check

    import glob
    import importlib.util
    suite = unittest.TestSuite()
    for path in sorted(glob.glob(os.path.join(args.reference, "pyalign", "tests", "test_*.py"))):
        name = "pyalign_reference_tests." + os.path.splitext(os.path.basename(path))[0]
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        suite.addTests(unittest.defaultTestLoader.loadTestsFromModule(mod))
    result = unittest.TextTestRunner(verbosity=2).run(suite)
    if not result.wasSuccessful():
        raise SystemExit("the reference's own tests FAIL on the oracle")

    used = sorted({c["call"] for c in rec.checks})
    remap = {old: new for new, old in enumerate(used)}
    calls = []
    for c in rec.calls:
        if c["id"] in remap:
            c = dict(c)
            c["id"] = remap[c["id"]]
            calls.append(c)
    checks = [dict(k, call=remap[k["call"]]) for k in rec.checks]
    doc = {
        "source": "pyalign 0.4.4 pyalign/tests/*.py, replayed on oracle/pa_oracle.cpp",
        "tests_run": result.testsRun,
        "calls": calls,
        "checks": checks,
    }
    with open(args.out, "w") as f:
        json.dump(doc, f, indent=1)
    print(f"wrote {args.out}: {len(calls)} native calls, {len(checks)} checked results, "
          f"{result.testsRun} reference tests passed on the oracle")


if __name__ == "__main__":
    main()
