"""Replay recorded native ``solve_*`` calls on any module with pyalign's native API.

The fixtures in tests/golden/reference_tests.json hold the arrays that crossed the
reference's Python/C++ boundary (pyalign/solve.py:342-469 -> factory.h:414-508) while the
reference's own unit tests ran.  This helper rebuilds the options dict that
pyalign/solve.py:173-196 would pass, re-packs the lanes to the target module's
``batch_size`` and calls the same method, so the oracle and the GPU module can be checked
against the same calls.
"""

import json
import os
import types

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_tests.json")


def load_golden():
    with open(GOLDEN) as f:
        return json.load(f)


class RecordedGap:
    """Stand-in for a pyalign.gaps.GapCost with the recorded special case or cost vector."""

    def __init__(self, rec):
        self._rec = rec

    def to_special_case(self):
        r = self._rec
        if r["kind"] == "linear":
            return {"linear": r["w"]}
        if r["kind"] == "affine":
            # gaps.py:169-182 hands (open - extend, extend); the native side flips it
            return {"affine": (r["v"], r["u"])}
        return {}

    def costs(self, n):
        c = np.asarray(self._rec["costs"], dtype=np.float32)
        if c.shape[0] != n:
            raise ValueError(f"recorded {c.shape[0]} costs, asked for {n}")
        return c


def make_options(alg, rec_options):
    o = rec_options
    d = {
        "solver": alg.Type(o["type"]) if hasattr(alg.Type, "__call__") else o["type"],
        "direction": alg.Direction(o["direction"]),
        "batch": o["batch"],
        "return_dup": o["return_dup"],
        "locality": alg.Locality(o["locality"]),
        "codomain": types.SimpleNamespace(detail=alg.Detail(o["detail"]), count=alg.Count(o["count"])),
        "gap_cost": {"s": RecordedGap(o["gap_s"]), "t": RecordedGap(o["gap_t"])},
    }
    return d


def make_solver(alg, call, batch=None):
    mod = alg.m16 if call["index_bits"] == 16 else alg.m32
    d = make_options(alg, call["options"])
    if batch is not None:
        d["batch"] = batch
    opts = mod.create_options(d)
    return mod.create_solver(call["cap"][0], call["cap"][1], opts)


def repack(call, batch_size):
    """Inputs of a recorded call with the lane axis re-sized to batch_size."""
    args = call["args"]
    length = np.asarray(args["len"], dtype=np.uint16)
    n = length.shape[1]
    assert n <= batch_size, (n, batch_size)
    ln = np.zeros((2, batch_size), dtype=np.uint16)
    ln[:, :n] = length
    out = {}
    if "a" in args:
        for k in ("a", "b"):
            x = np.asarray(args[k], dtype=np.uint32)
            y = np.zeros((batch_size, x.shape[1]), dtype=np.uint32)
            y[:n] = x
            out[k] = y
    if "sim" in args:
        sim = np.asarray(args["sim"], dtype=np.float32)
        if sim.ndim == 3:
            y = np.zeros(sim.shape[:2] + (batch_size,), dtype=np.float32)
            y[:, :, :n] = sim
            out["sim"] = y
        else:
            out["sim"] = sim
    if "eq" in args:
        out["eq"] = args["eq"]
        out["ne"] = args["ne"]
    out["len"] = ln
    return out, n


def call_args(method, packed):
    if method.startswith("solve_indexed_for"):
        return (packed["a"], packed["b"], packed["sim"], packed["len"])
    if method.startswith("solve_binary_for"):
        return (packed["a"], packed["b"], packed["eq"], packed["ne"], packed["len"])
    return (packed["sim"], packed["len"])


def run_call(alg, call):
    """Run a recorded call on `alg`; returns per-lane results (lanes of the recording)."""
    solver = make_solver(alg, call)
    packed, n = repack(call, solver.batch_size)
    res = getattr(solver, call["method"])(*call_args(call["method"], packed))
    return solver, res, n


def drain(iterator):
    out = []
    while True:
        x = iterator.next()
        if x is None:
            return out
        out.append(x)


def edges_of(alignment):
    s_to_t = np.asarray(alignment.s_to_t)
    i = np.nonzero(s_to_t >= 0)[0]
    return np.column_stack([i, s_to_t[i]]).tolist()
