"""Seeded problem generators and a call-for-call comparator (GPU module vs oracle).

The gap objects restate the cost formulas of pyalign/gaps.py:120-225 (LinearGapCost,
AffineGapCost, LogarithmicGapCost) so that the options dicts built here are the ones
pyalign/solve.py:173-196 would hand to the native module.
"""

import types

import numpy as np


class Gap:
    def __init__(self, kind, a=0.0, b=0.0):
        self.kind, self.a, self.b = kind, a, b

    def __repr__(self):
        return f"Gap({self.kind},{self.a},{self.b})"

    def to_special_case(self):
        if self.kind == "linear":
            return {"linear": self.a}
        if self.kind == "affine":  # AffineGapCost(open=a, extend=b): u = open - extend, v = extend
            return {"affine": (self.a - self.b, self.b)}
        return {}

    def costs(self, n):
        if self.kind == "linear":
            return np.linspace(0., (n - 1) * self.a, n, dtype=np.float32)
        if self.kind == "affine":
            w = (self.a - self.b) + np.linspace(0., (n - 1) * self.b, n, dtype=np.float32)
            w[0] = 0
            return w.astype(np.float32)
        # logarithmic: u + v ln(k)
        w = np.full((n,), self.a, dtype=np.float32)
        w[1:] += self.b * np.log(np.arange(1, n), dtype=np.float32)
        w[0] = 0
        return w


def options(alg, *, dtw=False, locality="global", direction="maximize", detail="alignment",
            count="one", gap=None, batch=True, batch_size=None, return_dup=False):
    d = {
        "solver": alg.Type.DTW if dtw else alg.Type.ALIGNMENT,
        "direction": alg.Direction.__members__[direction.upper()],
        "batch": batch,
        "return_dup": return_dup,
        "locality": alg.Locality.__members__[locality.upper()],
        "codomain": types.SimpleNamespace(detail=alg.Detail.__members__[detail.upper()],
                                          count=alg.Count.__members__[count.upper()]),
        "gap_cost": gap,
    }
    if batch_size is not None:
        d["batch_size"] = batch_size
    return d


def random_pairs(rng, n, lo, hi, alphabet=4, related=0.5):
    """n pairs of code sequences with lengths in [lo, hi]; some t are mutated copies of s."""
    pairs = []
    for _ in range(n):
        ls = int(rng.integers(lo, hi + 1))
        s = rng.integers(0, alphabet, size=ls).astype(np.uint32)
        if ls and rng.random() < related:
            t = s.copy()
            for _k in range(max(1, ls // 10)):
                op = rng.integers(0, 3)
                pos = int(rng.integers(0, max(len(t), 1)))
                if op == 0 and len(t):
                    t[pos % len(t)] = rng.integers(0, alphabet)
                elif op == 1:
                    t = np.insert(t, pos, rng.integers(0, alphabet))
                elif len(t) > 1:
                    t = np.delete(t, pos % len(t))
            t = t[:hi] if len(t) > hi else t
        else:
            t = rng.integers(0, alphabet, size=int(rng.integers(lo, hi + 1))).astype(np.uint32)
        pairs.append((s.astype(np.uint32), np.asarray(t, dtype=np.uint32)))
    return pairs


def pack(pairs, batch):
    n_s = max([len(s) for s, _ in pairs] + [1])
    n_t = max([len(t) for _, t in pairs] + [1])
    a = np.zeros((batch, n_s), dtype=np.uint32)
    b = np.zeros((batch, n_t), dtype=np.uint32)
    ln = np.zeros((2, batch), dtype=np.uint16)
    for k, (s, t) in enumerate(pairs):
        a[k, :len(s)] = s
        b[k, :len(t)] = t
        ln[0, k], ln[1, k] = len(s), len(t)
    return a, b, ln


def dense_of(a, b, ln, table):
    """(n_s, n_t, batch) lane-minor similarity built from a table (solve.py:342-379 layout)."""
    batch = a.shape[0]
    sim = np.zeros((a.shape[1], b.shape[1], batch), dtype=np.float32)
    for k in range(batch):
        sim[:, :, k] = table[np.ix_(a[k], b[k])]
    return sim


def call(alg, opts, cap, method, form, a, b, ln, table=None, eq=1.0, ne=-1.0, sim=None, bits=16):
    mod = alg.m16 if bits == 16 else alg.m32
    solver = mod.create_solver(cap[0], cap[1], mod.create_options(dict(opts)))
    name = {"dense": "solve_for_", "indexed": "solve_indexed_for_", "binary": "solve_binary_for_"}[form] + method
    fn = getattr(solver, name)
    if form == "dense":
        return solver, fn(sim, ln)
    if form == "indexed":
        return solver, fn(a, b, table, ln)
    return solver, fn(a, b, eq, ne, ln)


def drain(it, cap=60):
    out = []
    while len(out) < cap:
        x = it.next()
        if x is None:
            break
        out.append(x)
    return out


def _eq_arrays(x, y):
    x, y = np.asarray(x), np.asarray(y)
    if x.shape != y.shape:
        return False
    if x.dtype.kind == "f":
        return bool(np.all((x == y) | (np.isnan(x) & np.isnan(y))))
    return bool(np.array_equal(x, y))


def same_alignment(g, o):
    return (g.score == o.score or (np.isnan(g.score) and np.isnan(o.score))) and \
        _eq_arrays(g.s_to_t, o.s_to_t) and _eq_arrays(g.t_to_s, o.t_to_s)


def same_solution(g, o):
    if not _eq_arrays(g.values, o.values):
        return "values"
    if not _eq_arrays(g.traceback_as_matrix, o.traceback_as_matrix):
        return "traceback_as_matrix"
    ge, oe = g.traceback_as_edges, o.traceback_as_edges
    if len(ge) != len(oe) or not all(_eq_arrays(x, y) for x, y in zip(ge, oe)):
        return "traceback_as_edges"
    if (g.path is None) != (o.path is None) or (g.path is not None and not _eq_arrays(g.path, o.path)):
        return "path"
    if g.score != o.score:
        return "score"
    if (g.alignment is None) != (o.alignment is None):
        return "alignment presence"
    if g.alignment is not None and not same_alignment(g.alignment, o.alignment):
        return "alignment"
    if g.traceback_has_max_degree_1 != o.traceback_has_max_degree_1:
        return "max_degree_1"
    ga, oa = g.algorithm, o.algorithm
    if (ga is None) != (oa is None) or (ga is not None and (ga.name, ga.runtime, ga.memory) != (oa.name, oa.runtime, oa.memory)):
        return "algorithm"
    return None


def compare(method, gpu_out, ora_out, n, iter_cap=60):
    """Returns None when equal, else a description of the first difference."""
    if method == "score":
        g, o = np.asarray(gpu_out)[:n], np.asarray(ora_out)[:n]
        if not _eq_arrays(g, o):
            bad = np.nonzero(~((g == o) | (np.isnan(g) & np.isnan(o))))[0]
            return f"scores differ at lanes {bad[:10].tolist()}: gpu {g[bad[:5]]} oracle {o[bad[:5]]}"
        return None
    for k in range(n):
        g, o = gpu_out[k], ora_out[k]
        if method == "alignment":
            if not same_alignment(g, o):
                return f"lane {k}: alignment gpu ({g.score}, {g.s_to_t}) oracle ({o.score}, {o.s_to_t})"
        elif method == "alignment_iterator":
            gl, ol = drain(g, iter_cap), drain(o, iter_cap)
            if len(gl) != len(ol):
                return f"lane {k}: {len(gl)} vs {len(ol)} alignments"
            for q, (x, y) in enumerate(zip(gl, ol)):
                if not same_alignment(x, y):
                    return f"lane {k} item {q}: gpu ({x.score}, {x.s_to_t}) oracle ({y.score}, {y.s_to_t})"
        elif method == "solution":
            d = same_solution(g, o)
            if d:
                return f"lane {k}: solution differs in {d}"
        else:
            gl, ol = drain(g, 8), drain(o, 8)
            if len(gl) != len(ol):
                return f"lane {k}: {len(gl)} vs {len(ol)} solutions"
            for q, (x, y) in enumerate(zip(gl, ol)):
                d = same_solution(x, y)
                if d:
                    return f"lane {k} item {q}: solution differs in {d}"
    return None
