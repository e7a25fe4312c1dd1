"""Oracle-backed stand-in for pyalign's native ``algorithm`` module -- TEST INFRASTRUCTURE.

It exposes the same names as the pybind11 module registered in
pyalign/algorithm/pyalign.h:17-102 and module.cpp:7-18 (enums, ``m16``/``m32`` with
``create_options``/``create_solver``, ``Solver`` with the 15 ``solve_*`` methods,
``Alignment``, ``AlignmentIterator``, ``Solution``, ``SolutionIterator``), but every pair is
solved by the scalar C++ restatement in ``oracle/pa_oracle.cpp``, one pair at a time.

It exists so that (1) the reference's own Python package and unit tests run on the oracle
(which pins the oracle to the reference's golden vectors) and (2) the GPU module can be
compared with it call for call.  Only tests, the smoke check and bench.py's CPU baseline
import it.
"""

import ctypes
import enum
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpa_oracle.so")


def build(force=False):
    """Compile the oracle shared library with g++ (Makefile in this directory)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "pa_oracle.cpp"))):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Options(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32), ("direction", ctypes.c_int32), ("detail", ctypes.c_int32),
        ("count", ctypes.c_int32), ("locality", ctypes.c_int32), ("remove_dup", ctypes.c_int32),
        ("gap_kind", ctypes.c_int32),
        ("linear_s", ctypes.c_float), ("linear_t", ctypes.c_float),
        ("affine_u_s", ctypes.c_float), ("affine_v_s", ctypes.c_float),
        ("affine_u_t", ctypes.c_float), ("affine_v_t", ctypes.c_float),
        ("general_s", ctypes.POINTER(ctypes.c_float)), ("general_t", ctypes.POINTER(ctypes.c_float)),
        ("cap_s", ctypes.c_int32), ("cap_t", ctypes.c_int32),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        lib.pao_solve.restype = P
        lib.pao_solve.argtypes = [ctypes.POINTER(_Options), ctypes.c_int32, ctypes.c_int32,
                                  ctypes.POINTER(ctypes.c_float)]
        lib.pao_free.argtypes = [P]
        lib.pao_goal.argtypes = [P]
        lib.pao_layer_count.argtypes = [P]
        lib.pao_next.restype = ctypes.c_int32
        lib.pao_next.argtypes = [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32),
                                 ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        lib.pao_worst.restype = ctypes.c_float
        lib.pao_worst.argtypes = [P]
        lib.pao_values.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)]
        lib.pao_tb_matrix.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        lib.pao_tb_edges.restype = ctypes.c_int64
        lib.pao_tb_edges.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
        _lib = lib
    return _lib


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


# --- enums (enum.h:8-33, pyalign.h:80-102) ---

class Type(enum.IntEnum):
    ALIGNMENT = 0
    DTW = 1


class Direction(enum.IntEnum):
    MINIMIZE = 0
    MAXIMIZE = 1


class Detail(enum.IntEnum):
    SCORE = 0
    ALIGNMENT = 1
    SOLUTION = 2


class Count(enum.IntEnum):
    ONE = 0
    ALL = 1


class Locality(enum.IntEnum):
    LOCAL = 0
    GLOBAL = 1
    SEMIGLOBAL = 2


class Algorithm:
    """Solver metadata (solver.h:154-177)."""

    def __init__(self, name, runtime, memory):
        self._name, self._runtime, self._memory = name, runtime, memory

    name = property(lambda self: self._name)
    runtime = property(lambda self: self._runtime)
    memory = property(lambda self: self._memory)


# --- options (options.h:9-117, factory.h:33-108) ---

def _gap_spec(g):
    """GapCostOptions (factory.h:33-65) for one side."""
    if g is None:
        return ("linear", np.float32(0.0))
    sc = g.to_special_case()
    if "affine" in sc:
        t = sc["affine"]
        # factory.h:48-52 flips (u, v) into Gotoh's w(k) = u k + v
        return ("affine", (np.float32(t[1]), np.float32(t[0])))
    if "linear" in sc:
        return ("linear", np.float32(sc["linear"]))
    return ("general", g)


class Options:
    def __init__(self, d, index_bits):
        self._d = d
        self.index_bits = index_bits
        self.type = Type(int(d["solver"]))
        self.batch = bool(d["batch"])
        self.direction = Direction(int(d["direction"]))
        self.remove_dup = not bool(d["return_dup"])
        self.batch_size = d.get("batch_size") if hasattr(d, "get") else None
        if self.type == Type.ALIGNMENT:
            cod = d["codomain"]
            self.detail = Detail(int(cod.detail))
            self.count = Count(int(cod.count))
            self.locality = Locality(int(d["locality"])) if "locality" in d else Locality.LOCAL
            gc = d["gap_cost"] if "gap_cost" in d else None
            if isinstance(gc, dict):
                gs, gt = gc.get("s"), gc.get("t")
            else:
                gs, gt = gc, gc
            self.gap_s, self.gap_t = _gap_spec(gs), _gap_spec(gt)
        else:
            self.detail, self.count, self.locality = Detail.ALIGNMENT, Count.ONE, Locality.GLOBAL
            self.gap_s = self.gap_t = ("linear", np.float32(0.0))

    def to_dict(self):
        return self._d


def _general_costs(spec, n):
    kind, val = spec
    if kind == "general":
        c = np.asarray(val.costs(n), dtype=np.float32)
        if c.shape != (n,):
            raise ValueError(f"expected gap cost tensor length of {n}, got {c.shape[0]}")
        return c
    if kind == "linear" and val == 0:
        return np.zeros((n,), dtype=np.float32)
    raise ValueError("mixed special-case gap costs have no defined general form")


# --- results (factory.h:130-193, 250-352) ---

class Alignment:
    def __init__(self, ls, lt, score, mp, index_dtype, has):
        self._ls, self._lt = ls, lt
        self._score = float(np.float32(score))
        self._s_to_t = None
        self._t_to_s = None
        mp = np.asarray(mp, dtype=index_dtype)
        if not has:
            mp = np.full((min(ls, lt),), -1, dtype=index_dtype)
        if ls <= lt:
            self._s_to_t = mp
        else:
            self._t_to_s = mp
        self._dtype = index_dtype

    @property
    def score(self):
        return self._score

    @staticmethod
    def _invert(src, n, dtype):
        out = np.full((n,), -1, dtype=dtype)
        idx = np.nonzero(src >= 0)[0]
        out[src[idx]] = idx
        return out

    @property
    def s_to_t(self):
        if self._s_to_t is None:
            self._s_to_t = self._invert(self._t_to_s, self._ls, self._dtype)
        return self._s_to_t

    @property
    def t_to_s(self):
        if self._t_to_s is None:
            self._t_to_s = self._invert(self._s_to_t, self._lt, self._dtype)
        return self._t_to_s


def _algorithm_meta(opts, gap_kind):
    if opts.type == Type.DTW:
        return Algorithm("DTW", "n^2", "n^2")
    if gap_kind == 0:
        return Algorithm("Needleman-Wunsch" if opts.locality == Locality.GLOBAL else "Smith-Waterman",
                         "n^2", "n^2")
    if gap_kind == 1:
        return Algorithm("Gotoh", "n^2", "n^2")
    return Algorithm("Waterman-Smith-Beyer", "n^3", "n^2")


class _Pair:
    """One solved pair held by the oracle."""

    def __init__(self, solver, ls, lt, sim):
        self.solver = solver
        self.ls, self.lt = ls, lt
        sim = np.ascontiguousarray(sim, dtype=np.float32).reshape(ls, lt) if ls * lt else \
            np.zeros((max(ls, 1), max(lt, 1)), dtype=np.float32)
        self._ptr = _load().pao_solve(ctypes.byref(solver._copts), ls, lt, _fptr(sim))

    def __del__(self):
        if getattr(self, "_ptr", None):
            _load().pao_free(self._ptr)
            self._ptr = None

    def next(self):
        lib = _load()
        sc = ctypes.c_float(0)
        mp = np.full((min(self.ls, self.lt),), -1, dtype=np.int32)
        path = np.zeros((self.ls + self.lt + 4, 2), dtype=np.int32)
        n = ctypes.c_int32(0)
        ok = lib.pao_next(self._ptr, ctypes.byref(sc), _iptr(mp), _iptr(path), ctypes.byref(n))
        if not ok:
            return None
        return float(sc.value), mp, path[:n.value].copy()

    def worst(self):
        return float(_load().pao_worst(self._ptr))

    def layers(self):
        return int(_load().pao_layer_count(self._ptr))

    def values(self, k):
        out = np.zeros((self.ls + 1, self.lt + 1), dtype=np.float32)
        _load().pao_values(self._ptr, k, _fptr(out))
        return out

    def tb_matrix(self, k):
        out = np.zeros((self.ls + 1, self.lt + 1, 2), dtype=np.int32)
        _load().pao_tb_matrix(self._ptr, k, _iptr(out))
        return out

    def tb_edges(self, k):
        lib = _load()
        n = int(lib.pao_tb_edges(self._ptr, k, None))
        out = np.zeros((n, 2, 2), dtype=np.int32)
        if n:
            lib.pao_tb_edges(self._ptr, k, _iptr(out))
        return out


def _to_index(a, dtype):
    a = np.asarray(a)
    lo = np.iinfo(dtype).min
    return np.where(a == np.iinfo(np.int32).min, lo, a).astype(dtype)


class Solution:
    def __init__(self, pair, nlayers, max_degree_1, res, algorithm, index_dtype):
        self._values = np.stack([pair.values(k) for k in range(nlayers)])
        self._tbm = _to_index(np.stack([pair.tb_matrix(k) for k in range(nlayers)]), index_dtype)
        self._edges = [_to_index(pair.tb_edges(k), index_dtype) for k in range(nlayers)]
        self._deg1 = max_degree_1
        self._algorithm = algorithm
        if res is None:
            self._score = None
            self._alignment = None
            self._path = None
        else:
            sc, mp, path = res
            self._alignment = Alignment(pair.ls, pair.lt, sc, mp, index_dtype, True)
            self._score = self._alignment.score
            self._path = _to_index(path, index_dtype)

    values = property(lambda self: self._values)
    traceback_has_max_degree_1 = property(lambda self: self._deg1)
    traceback_as_matrix = property(lambda self: self._tbm)
    traceback_as_edges = property(lambda self: list(self._edges))
    path = property(lambda self: self._path)
    score = property(lambda self: self._score)
    alignment = property(lambda self: self._alignment)
    algorithm = property(lambda self: self._algorithm)


class AlignmentIterator:
    def __init__(self, pair, index_dtype):
        self._pair, self._dtype = pair, index_dtype

    def next(self):
        r = self._pair.next()
        if r is None:
            return None
        sc, mp, _ = r
        return Alignment(self._pair.ls, self._pair.lt, sc, mp, self._dtype, True)


class SolutionIterator:
    def __init__(self, pair, index_dtype, max_degree_1):
        self._pair, self._dtype, self._deg1 = pair, index_dtype, max_degree_1

    def next(self):
        r = self._pair.next()
        if r is None:
            return None
        return Solution(self._pair, 1, self._deg1, r, None, self._dtype)


class Solver:
    """Oracle solver with the reference's Solver interface (factory.h:414-508)."""

    LANES = 4  # 128-bit SIMD lanes of float32 on the aarch64 host (solver.h:394-395)

    def __init__(self, max_len_s, max_len_t, options):
        self._opts = options
        idx = np.int16 if options.index_bits == 16 else np.int32
        self._index_dtype = idx
        lim = np.iinfo(idx).max >> 1
        for name, n in (("s", max_len_s), ("t", max_len_t)):
            if n > lim:
                raise RuntimeError(
                    f"requested maximum length {n} for {name} exceeds maximum supported "
                    f"sequence length in this implementation {lim}")
        self._cap_s, self._cap_t = int(max_len_s), int(max_len_t)
        self._batch_size = (int(options.batch_size or self.LANES)) if options.batch else 1
        o = options
        kinds = (o.gap_s[0], o.gap_t[0])
        if o.type == Type.DTW:
            gap_kind = 0
        elif kinds == ("linear", "linear"):
            gap_kind = 0
        elif kinds == ("affine", "affine"):
            gap_kind = 1
        else:
            gap_kind = 2
        self._gap_kind = gap_kind
        c = _Options()
        c.type, c.direction = int(o.type), int(o.direction)
        c.detail, c.count, c.locality = int(o.detail), int(o.count), int(o.locality)
        c.remove_dup, c.gap_kind = int(o.remove_dup), gap_kind
        if gap_kind == 0:
            c.linear_s, c.linear_t = float(o.gap_s[1]), float(o.gap_t[1])
        elif gap_kind == 1:
            c.affine_u_s, c.affine_v_s = float(o.gap_s[1][0]), float(o.gap_s[1][1])
            c.affine_u_t, c.affine_v_t = float(o.gap_t[1][0]), float(o.gap_t[1][1])
        else:
            self._gen_s = _general_costs(o.gap_s, self._cap_s + 1)
            self._gen_t = _general_costs(o.gap_t, self._cap_t + 1)
            c.general_s, c.general_t = _fptr(self._gen_s), _fptr(self._gen_t)
        c.cap_s, c.cap_t = self._cap_s, self._cap_t
        self._copts = c
        self._algorithm = _algorithm_meta(o, gap_kind)

    @property
    def options(self):
        return self._opts.to_dict()

    @property
    def batch_size(self):
        return self._batch_size

    # --- input forms (factory.h:513-680) ---

    def _check_len(self, length):
        length = np.asarray(length)
        if length.ndim != 2 or length.shape[0] != 2 or length.shape[1] != self._batch_size:
            raise ValueError(f"m_length has shape {length.shape}, expected (2, {self._batch_size})")
        return length.astype(np.int64)

    def _check_batch(self, given):
        if given != self._batch_size:
            raise ValueError(f"problem of batch size {given} given to solver that was "
                             f"configured to batch size {self._batch_size}")

    def _check_cap(self, ls, lt):
        if ls > self._cap_s:
            raise RuntimeError(f"sequence s of length {ls} exceeds configured maximum length {self._cap_s}")
        if lt > self._cap_t:
            raise RuntimeError(f"sequence t of length {lt} exceeds configured maximum length {self._cap_t}")

    def _pairs_dense(self, sim, length):
        sim = np.asarray(sim, dtype=np.float32)
        self._check_batch(sim.shape[2])
        length = self._check_len(length)
        self._check_cap(sim.shape[0], sim.shape[1])
        out = []
        for k in range(self._batch_size):
            ls, lt = self._lane_lengths(length, k, sim.shape[0], sim.shape[1])
            out.append(_Pair(self, ls, lt, sim[:ls, :lt, k]))
        return out

    @staticmethod
    def _lane_lengths(length, k, n_s, n_t):
        """Lane k's lengths, clamped to the batch arrays: a partial batch's trailing lanes keep
        the lengths of an earlier, larger batch (solve.py:382-396 rewrites only the lanes it
        fills); the reference computes them over stale array contents and pyalign discards
        their results (solve.py:554-560), so any value serves -- clamping keeps them in the
        arrays."""
        return min(int(length[0, k]), n_s), min(int(length[1, k]), n_t)

    def _pairs_indexed(self, a, b, sim, length):
        a, b = np.asarray(a), np.asarray(b)
        sim = np.asarray(sim, dtype=np.float32)
        self._check_batch(a.shape[0])
        self._check_batch(b.shape[0])
        if a.size and a.max() >= sim.shape[0]:
            raise ValueError("out of bounds index in a")
        if b.size and b.max() >= sim.shape[1]:
            raise ValueError("out of bounds index in b")
        length = self._check_len(length)
        self._check_cap(a.shape[1], b.shape[1])
        out = []
        for k in range(self._batch_size):
            ls, lt = self._lane_lengths(length, k, a.shape[1], b.shape[1])
            out.append(_Pair(self, ls, lt, sim[np.ix_(a[k, :ls], b[k, :lt])]))
        return out

    def _pairs_binary(self, a, b, eq, ne, length):
        a, b = np.asarray(a), np.asarray(b)
        self._check_batch(a.shape[0])
        self._check_batch(b.shape[0])
        length = self._check_len(length)
        self._check_cap(a.shape[1], b.shape[1])
        eq, ne = np.float32(eq), np.float32(ne)
        out = []
        for k in range(self._batch_size):
            ls, lt = self._lane_lengths(length, k, a.shape[1], b.shape[1])
            m = a[k, :ls][:, None] == b[k, :lt][None, :]
            out.append(_Pair(self, ls, lt, np.where(m, eq, ne).astype(np.float32)))
        return out

    # --- codomains (factory.h:699-808) ---

    def _for_score(self, pairs):
        out = np.zeros((self._batch_size,), dtype=np.float32)
        for k, p in enumerate(pairs):
            r = p.next()
            out[k] = r[0] if r is not None else p.worst()
        return out

    def _for_alignment(self, pairs):
        res = []
        for p in pairs:
            r = p.next()
            if r is None:
                res.append(Alignment(p.ls, p.lt, p.worst(), [], self._index_dtype, False))
            else:
                res.append(Alignment(p.ls, p.lt, r[0], r[1], self._index_dtype, True))
        return tuple(res)

    def _for_alignment_iterator(self, pairs):
        return tuple(AlignmentIterator(p, self._index_dtype) for p in pairs)

    def _max_degree_1(self):
        return self._opts.type == Type.DTW or self._opts.count == Count.ONE

    def _for_solution(self, pairs):
        return tuple(Solution(p, p.layers(), self._max_degree_1(), p.next(), self._algorithm,
                              self._index_dtype) for p in pairs)

    def _for_solution_iterator(self, pairs):
        return tuple(SolutionIterator(p, self._index_dtype, self._max_degree_1()) for p in pairs)

    def solve_for_score(self, sim, length):
        return self._for_score(self._pairs_dense(sim, length))

    def solve_indexed_for_score(self, a, b, sim, length):
        return self._for_score(self._pairs_indexed(a, b, sim, length))

    def solve_binary_for_score(self, a, b, eq, ne, length):
        return self._for_score(self._pairs_binary(a, b, eq, ne, length))

    def solve_for_alignment(self, sim, length):
        return self._for_alignment(self._pairs_dense(sim, length))

    def solve_for_alignment_iterator(self, sim, length):
        return self._for_alignment_iterator(self._pairs_dense(sim, length))

    def solve_indexed_for_alignment(self, a, b, sim, length):
        return self._for_alignment(self._pairs_indexed(a, b, sim, length))

    def solve_indexed_for_alignment_iterator(self, a, b, sim, length):
        return self._for_alignment_iterator(self._pairs_indexed(a, b, sim, length))

    def solve_binary_for_alignment(self, a, b, eq, ne, length):
        return self._for_alignment(self._pairs_binary(a, b, eq, ne, length))

    def solve_binary_for_alignment_iterator(self, a, b, eq, ne, length):
        return self._for_alignment_iterator(self._pairs_binary(a, b, eq, ne, length))

    def solve_for_solution(self, sim, length):
        return self._for_solution(self._pairs_dense(sim, length))

    def solve_for_solution_iterator(self, sim, length):
        return self._for_solution_iterator(self._pairs_dense(sim, length))

    def solve_indexed_for_solution(self, a, b, sim, length):
        return self._for_solution(self._pairs_indexed(a, b, sim, length))

    def solve_indexed_for_solution_iterator(self, a, b, sim, length):
        return self._for_solution_iterator(self._pairs_indexed(a, b, sim, length))

    def solve_binary_for_solution(self, a, b, eq, ne, length):
        return self._for_solution(self._pairs_binary(a, b, eq, ne, length))

    def solve_binary_for_solution_iterator(self, a, b, eq, ne, length):
        return self._for_solution_iterator(self._pairs_binary(a, b, eq, ne, length))


class _IndexModule:
    """The ``m16``/``m32`` submodules (module.cpp:10-14)."""

    def __init__(self, bits):
        self._bits = bits
        self.Solver = Solver
        self.Alignment = Alignment
        self.AlignmentIterator = AlignmentIterator
        self.Solution = Solution
        self.SolutionIterator = SolutionIterator
        self.Options = Options

    def create_options(self, d):
        return Options(dict(d), self._bits)

    def create_solver(self, max_len_s, max_len_t, options):
        return Solver(max_len_s, max_len_t, options)


m16 = _IndexModule(16)
m32 = _IndexModule(32)


# --- threaded batch helpers of the oracle (indexed form) ---

def _batch_args(a, b, ls, lt, table):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    ls = np.ascontiguousarray(ls, dtype=np.int32)
    lt = np.ascontiguousarray(lt, dtype=np.int32)
    table = np.ascontiguousarray(table, dtype=np.float32)
    return a, b, ls, lt, table


def batch_alignments(solver, a, b, table, ls, lt, threads=None):
    """Score and one alignment map per pair of the indexed form on `threads` host threads,
    each pair as one lane of Solver::alignment (solver.h:2610-2630), with the options of an
    oracle `solver`.  Returns (scores f32[n], maps i32 concatenated at offsets, offsets
    i64[n + 1] = prefix sums of min(|s|, |t|), cells)."""
    lib = _load()
    a, b, ls, lt, table = _batch_args(a, b, ls, lt, table)
    n = len(ls)
    sizes = np.minimum(ls, lt).astype(np.int64)
    offs = np.zeros(n + 1, np.int64)
    offs[1:] = np.cumsum(sizes)
    maps = np.zeros(int(offs[-1]) + 1, np.int32)
    scores = np.zeros(n, np.float32)
    vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    lib.pao_batch_alignments.restype = i64
    lib.pao_batch_alignments.argtypes = [vp, i32, vp, vp, vp, i64, vp, i64, vp, i32, i32, vp, vp, vp]
    cells = lib.pao_batch_alignments(
        ctypes.addressof(solver._copts), n, ls.ctypes.data, lt.ctypes.data, a.ctypes.data, a.shape[1],
        b.ctypes.data, b.shape[1], table.ctypes.data, table.shape[1], int(threads or os.cpu_count() or 1),
        scores.ctypes.data, maps.ctypes.data, offs.ctypes.data)
    return scores, maps[:int(offs[-1])], offs, int(cells)


def batch_scores_lean(solver, a, b, table, ls, lt, threads=None):
    """Scores of the indexed form with two rows per layer (memory O(|t|) per pair, for pairs
    of 5000 x 10000 cells), linear or affine gaps, with the options of an oracle `solver`.
    Returns (scores f32[n], cells)."""
    lib = _load()
    a, b, ls, lt, table = _batch_args(a, b, ls, lt, table)
    n = len(ls)
    scores = np.zeros(n, np.float32)
    vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    lib.pao_batch_scores_lean.restype = i64
    lib.pao_batch_scores_lean.argtypes = [vp, i32, vp, vp, vp, i64, vp, i64, vp, i32, i32, vp]
    cells = lib.pao_batch_scores_lean(
        ctypes.addressof(solver._copts), n, ls.ctypes.data, lt.ctypes.data, a.ctypes.data, a.shape[1],
        b.ctypes.data, b.shape[1], table.ctypes.data, table.shape[1], int(threads or os.cpu_count() or 1),
        scores.ctypes.data)
    return scores, int(cells)


def batch_f64(S, ls, lt, *, dtw=False, locality="global", direction="maximize", open_=0.5, extend=0.1,
              threads=None):
    """The FP64 twin on a batch of float32 matrices S (B, n, m) (converted to double): global
    (or `locality`) affine Gotoh with open/extend, or DTW.  Returns (scores f64[B], scales
    f64[B]) where scale = sum |S| over the cells the optimal path adds + the path's gap cost."""
    lib = _load()
    S = np.ascontiguousarray(S, dtype=np.float32)
    ls = np.ascontiguousarray(ls, dtype=np.int32)
    lt = np.ascontiguousarray(lt, dtype=np.int32)
    B = len(ls)
    o = _Options()
    o.type = int(Type.DTW if dtw else Type.ALIGNMENT)
    o.direction = int(Direction.__members__[direction.upper()])
    o.detail, o.count, o.remove_dup = 1, 0, 1
    o.locality = int(Locality.__members__[locality.upper()])
    o.gap_kind = 0 if dtw else 1
    o.cap_s, o.cap_t = int(ls.max(initial=0)), int(lt.max(initial=0))
    gaps = np.zeros(6, np.float64)
    if not dtw:
        gaps[2] = gaps[4] = extend
        gaps[3] = gaps[5] = open_ - extend
    scores = np.zeros(B, np.float64)
    scales = np.zeros(B, np.float64)
    vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    lib.pao_batch_f64.restype = None
    lib.pao_batch_f64.argtypes = [vp, vp, i32, vp, vp, vp, i64, i64, i32, vp, vp]
    lib.pao_batch_f64(ctypes.addressof(o), gaps.ctypes.data, B, ls.ctypes.data, lt.ctypes.data, S.ctypes.data,
                      S.shape[1] * S.shape[2], S.shape[2], int(threads or os.cpu_count() or 1),
                      scores.ctypes.data, scales.ctypes.data)
    return scores, scales
