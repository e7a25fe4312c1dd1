"""Drop-in replacement for pyalign's native ``algorithm`` module, backed by the GB300 library.

pyalign 0.4.4 obtains its compute core as ``algorithm = import_algorithm()``
(pyalign/solve.py:18, pyalign/cpu.py:21-47), a pybind11 module whose names are registered
in pyalign/algorithm/pyalign.h:17-102 and module.cpp:7-18.  This module exports the same
names -- the enums, ``Algorithm``, and the ``m16``/``m32`` submodules with
``create_options``/``create_solver``, ``Solver`` (15 ``solve_*`` methods, ``batch_size``,
``options``), ``Alignment``, ``AlignmentIterator``, ``Solution``, ``SolutionIterator`` --
with the same argument meaning and errors (ValueError for std::invalid_argument,
RuntimeError for the length exceptions), over the C ABI of include/pyalign_gb300.h.

Every solve runs on the GPU.  If the library is not built or no CUDA device is present,
calls fail loudly; there is no CPU fallback.
"""

import collections.abc
import ctypes
import enum
import functools
import operator
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpyalign_gb300.so")

PA_OK, PA_ERR_INVALID_ARGUMENT, PA_ERR_LENGTH = 0, 1, 2
PA_ERR_UNSUPPORTED = 7

_c_i32, _c_i64, _c_f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float
_P = ctypes.c_void_p
_PF = ctypes.POINTER(ctypes.c_float)
_PI = ctypes.POINTER(ctypes.c_int32)
_PU = ctypes.POINTER(ctypes.c_uint32)
_PL = ctypes.POINTER(ctypes.c_int64)


class _Options(ctypes.Structure):
    _fields_ = [
        ("type", _c_i32), ("direction", _c_i32), ("detail", _c_i32), ("count", _c_i32),
        ("locality", _c_i32), ("remove_dup", _c_i32), ("batch", _c_i32), ("batch_size", _c_i32),
        ("index_bits", _c_i32), ("gap_kind", _c_i32),
        ("linear_s", _c_f32), ("linear_t", _c_f32),
        ("affine_u_s", _c_f32), ("affine_v_s", _c_f32), ("affine_u_t", _c_f32), ("affine_v_t", _c_f32),
        ("general_s", _PF), ("general_t", _PF),
    ]


class Batch(ctypes.Structure):
    """pa_batch of the C ABI (the bag-at-once form)."""
    _fields_ = [
        ("form", _c_i32), ("location", _c_i32), ("batch", _c_i64), ("n_s", _c_i64), ("n_t", _c_i64),
        ("a", _PU), ("b", _PU), ("sim", _PF), ("table", _PF), ("table_rows", _c_i64),
        ("table_cols", _c_i64), ("eq", _c_f32), ("ne", _c_f32), ("length", _PI),
    ]


_lib = None


def library_path():
    return _LIB_PATH


def lib():
    """The loaded C library (built by pyalign_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise ImportError(
                f"{_LIB_PATH} is missing: build it with `python -m pyalign_gb300.build` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(_LIB_PATH)
        L.pa_last_error.restype = ctypes.c_char_p
        L.pa_version.restype = ctypes.c_char_p
        L.pa_device_count.restype = _c_i32
        L.pa_solver_create.restype = _c_i32
        L.pa_solver_create.argtypes = [ctypes.POINTER(_Options), _c_i64, _c_i64, ctypes.POINTER(_P)]
        L.pa_solver_destroy.argtypes = [_P]
        L.pa_solver_batch_size.restype = _c_i32
        L.pa_solver_batch_size.argtypes = [_P]
        L.pa_solver_set_stream.argtypes = [_P, _P]
        L.pa_solver_last_timings.argtypes = [_P, _PF, _PI]
        L.pa_solver_last_plan.argtypes = [_P, _PI]
        L.pa_solver_last_bucket_widths.argtypes = [_P, _PI]
        dense = [_P, _PF, _c_i64, _c_i64, _c_i64, _PI]
        indexed = [_P, _PU, _PU, _c_i64, _c_i64, _c_i64, _PF, _c_i64, _c_i64, _PI]
        binary = [_P, _PU, _PU, _c_i64, _c_i64, _c_i64, _c_f32, _c_f32, _PI]
        for codomain in ("score", "alignment", "alignment_iterator", "solution", "solution_iterator"):
            out = [_PF] if codomain == "score" else [ctypes.POINTER(_P)]
            for prefix, args in (("pa_solve_for_", dense), ("pa_solve_indexed_for_", indexed),
                                 ("pa_solve_binary_for_", binary)):
                f = getattr(L, prefix + codomain)
                f.restype = _c_i32
                f.argtypes = args + out
        L.pa_solve_batch.restype = _c_i32
        L.pa_solve_batch.argtypes = [_P, ctypes.POINTER(Batch), _P, _P, _PL]
        L.pa_result_destroy.argtypes = [_P]
        L.pa_result_size.restype = _c_i64
        L.pa_result_size.argtypes = [_P]
        for f in ("pa_result_len_s", "pa_result_len_t"):
            getattr(L, f).restype = _c_i64
            getattr(L, f).argtypes = [_P, _c_i64]
        L.pa_result_has_alignment.restype = _c_i32
        L.pa_result_has_alignment.argtypes = [_P, _c_i64]
        L.pa_result_score.restype = _c_f32
        L.pa_result_score.argtypes = [_P, _c_i64]
        L.pa_result_alignment.argtypes = [_P, _c_i64, _PI]
        L.pa_result_export.argtypes = [_P, _PF, _PI, _PL]
        L.pa_result_lengths.restype = _c_i32
        L.pa_result_lengths.argtypes = [_P, _PI, _PI]
        L.pa_result_layers.restype = _c_i32
        L.pa_result_layers.argtypes = [_P, _c_i64]
        L.pa_result_max_degree_1.restype = _c_i32
        L.pa_result_max_degree_1.argtypes = [_P]
        L.pa_result_values.argtypes = [_P, _c_i64, _PF]
        L.pa_result_tb_matrix.argtypes = [_P, _c_i64, _PI]
        L.pa_result_tb_edges.restype = _c_i64
        L.pa_result_tb_edges.argtypes = [_P, _c_i64, _c_i32, _PI]
        L.pa_result_path.restype = _c_i64
        L.pa_result_path.argtypes = [_P, _c_i64, _PI]
        L.pa_result_algorithm.restype = ctypes.c_char_p
        L.pa_result_algorithm.argtypes = [_P, _c_i32]
        L.pa_result_iterator.argtypes = [_P, _c_i64, ctypes.POINTER(_P)]
        L.pa_iterator_next.restype = _c_i32
        L.pa_iterator_next.argtypes = [_P, _PF, _PI, _PI, _PL]
        L.pa_iterator_destroy.argtypes = [_P]
        L.pa_result_path_counts.argtypes = [_P, ctypes.POINTER(ctypes.c_uint64)]
        L.pa_result_first_alignments.argtypes = [_P, _c_i32, _PI, _PI, _PI, _PI]
        L.pa_solve_batch_result.argtypes = [_P, ctypes.POINTER(Batch), _PI, _PL, ctypes.POINTER(_P)]
        _lib = L
    return _lib


def check(status):
    if status == PA_OK:
        return
    msg = lib().pa_last_error().decode()
    if status == PA_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise RuntimeError(msg)


def _fp(a):
    return a.ctypes.data_as(_PF)


def _ip(a):
    return a.ctypes.data_as(_PI)


def _up(a):
    return a.ctypes.data_as(_PU)


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
    """Solver metadata (AlgorithmMetaData, solver.h:154-177; pyalign.h:72-78)."""

    def __init__(self, name, runtime, memory):
        self._v = (name, runtime, memory)

    name = property(lambda self: self._v[0])
    runtime = property(lambda self: self._v[1])
    memory = property(lambda self: self._v[2])


DEFAULT_BATCH_SIZE = int(os.environ.get("PYALIGN_GB300_BATCH_SIZE", "2048"))


def _gap_spec(g):
    """GapCostOptions (factory.h:33-65) for one side of the gap cost."""
    if g is None:
        return ("linear", np.float32(0.0))
    sc = g.to_special_case()
    if "affine" in sc:
        t = sc["affine"]
        # factory.h:42-52: (u, v) of w(k) = u + v k become Gotoh's w(k) = u' k + v'
        return ("affine", (np.float32(t[1]), np.float32(t[0])))
    if "linear" in sc:
        return ("linear", np.float32(sc["linear"]))
    return ("general", g)


class Options:
    """Parsed solver options (options.h:9-117)."""

    def __init__(self, d, index_bits):
        self._d = d
        self.index_bits = index_bits
        self.type = Type(int(d["solver"]))
        self.batch = bool(d["batch"])
        self.direction = Direction(int(d["direction"]))
        self.remove_dup = not bool(d["return_dup"])
        self.batch_size = int(d.get("batch_size", DEFAULT_BATCH_SIZE)) if hasattr(d, "get") else DEFAULT_BATCH_SIZE
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
        c = np.ascontiguousarray(val.costs(n), dtype=np.float32)
        if c.shape != (n,):
            raise ValueError(f"expected gap cost tensor length of {n}, got {c.shape[0]}")
        return c
    if kind == "linear":
        return (np.arange(n, dtype=np.float32) * np.float32(val)).astype(np.float32)
    u, v = val  # affine in Gotoh form
    w = (np.arange(n, dtype=np.float32) * u + v).astype(np.float32)
    w[0] = 0
    return w


# --- results ---

class _Result:
    """Owner of a pa_result handle (one solve call)."""

    __slots__ = ("ptr", "_path_counts", "_first")

    def __init__(self, ptr):
        self.ptr = ptr
        self._path_counts = None
        self._first = {}

    def __del__(self):
        if self.ptr and _lib is not None:
            _lib.pa_result_destroy(self.ptr)
            self.ptr = None


def _narrow(a, dtype):
    a = np.asarray(a)
    if dtype == np.int16:
        lo = np.iinfo(np.int16).min
        return np.where(a == np.iinfo(np.int32).min, lo, a).astype(np.int16)
    return a.astype(np.int32, copy=False)


class _Lanes(collections.abc.Sequence):
    """The per-lane results of one solve call -- the tuple the reference's methods return, one
    entry per lane (factory.h:699-808) -- with each entry made at its first access and kept:
    a call over 65,536 pairs returns without making 65,536 Python objects, and a consumer
    that walks the results (pyalign zips them with its problems, solve.py:374-379) makes each
    one once.  Indexing, negative indices, slices (as tuples), len() and iteration behave as
    on a tuple."""

    __slots__ = ("_make", "_items")

    def __init__(self, make, n):
        self._make = make
        self._items = [None] * n

    def __len__(self):
        return len(self._items)

    def __getitem__(self, k):
        if isinstance(k, slice):
            return tuple(self[i] for i in range(*k.indices(len(self._items))))
        n = len(self._items)
        k = operator.index(k)
        if k < 0:
            k += n
        if not 0 <= k < n:
            raise IndexError("result index out of range")
        x = self._items[k]
        if x is None:
            x = self._items[k] = self._make(k)
        return x

    def __iter__(self):
        for k in range(len(self._items)):
            yield self[k]

    def __repr__(self):
        return f"({', '.join(repr(x) for x in self)})"


class _AlignmentBatch:
    """The exported results of one solve call that lazy Alignment objects read from: all
    scores, all maps (int32; a lane's slice is narrowed to the index type when read),
    per-lane offsets and lengths."""

    __slots__ = ("scores", "maps", "offs", "sizes", "ls", "lt", "dtype")

    def __init__(self, scores, maps, offs, sizes, ls, lt, dtype):
        self.scores, self.maps, self.offs, self.sizes = scores, maps, offs, sizes
        self.ls, self.lt, self.dtype = ls, lt, dtype


class Alignment:
    """Alignment (factory.h:130-193): score plus s_to_t / t_to_s, -1 where unaligned.

    Alignments of a batch are created lazily (`_lazy`): they hold their batch and lane until
    a field is read, so a call returning 65,536 of them costs one export, not 65,536
    array conversions (pyalign wraps each one, solve.py:376-379)."""

    __slots__ = ("_ls", "_lt", "_score", "_s_to_t", "_t_to_s", "_dtype", "_src", "_k")

    def __init__(self, ls, lt, score, mp, index_dtype):
        self._src = None
        self._ls, self._lt = ls, lt
        self._score = float(score)
        self._dtype = index_dtype
        mp = _narrow(mp, index_dtype)
        if ls <= lt:
            self._s_to_t, self._t_to_s = mp, None
        else:
            self._s_to_t, self._t_to_s = None, mp

    @classmethod
    def _lazy(cls, batch, k):
        a = cls.__new__(cls)
        a._src = batch
        a._k = k
        return a

    def _load(self):
        b, k = self._src, self._k
        self._src = None
        self._ls, self._lt = int(b.ls[k]), int(b.lt[k])
        self._score = float(b.scores[k])
        self._dtype = b.dtype
        o = int(b.offs[k])
        mp = _narrow(b.maps[o:o + int(b.sizes[k])], b.dtype)
        if self._ls <= self._lt:
            self._s_to_t, self._t_to_s = mp, None
        else:
            self._s_to_t, self._t_to_s = None, mp

    @property
    def score(self):
        if self._src is not None:
            self._load()
        return self._score

    @staticmethod
    def _invert(src, n, dtype):  # factory.h:110-128
        out = np.full((n,), -1, dtype=dtype)
        idx = np.nonzero(src >= 0)[0]
        out[src[idx]] = idx
        return out

    @property
    def s_to_t(self):
        if self._src is not None:
            self._load()
        if self._s_to_t is None:
            self._s_to_t = self._invert(self._t_to_s, self._ls, self._dtype)
        return self._s_to_t

    @property
    def t_to_s(self):
        if self._src is not None:
            self._load()
        if self._t_to_s is None:
            self._t_to_s = self._invert(self._s_to_t, self._lt, self._dtype)
        return self._t_to_s


class Solution:
    """Solution (SolutionImpl, factory.h:284-352; core::Solution solver.h:2329-2507)."""

    def __init__(self, res, lane, ls, lt, dtype, step=None, algorithm=True, first=None):
        self._res, self._lane, self._ls, self._lt, self._dtype = res, lane, ls, lt, dtype
        self._step = step  # (score, map, path) of an iterator step, or None
        self._first = first  # all-optimal solver: () -> the result's FirstAlignments(k = 1, paths)
        self._with_algorithm = algorithm
        self._cache = {}

    def _get(self, key, fn):
        if key not in self._cache:
            self._cache[key] = fn()
        return self._cache[key]

    @property
    def values(self):
        def f():
            L = lib()
            k = L.pa_result_layers(self._res.ptr, self._lane)
            out = np.zeros((k, self._ls + 1, self._lt + 1), dtype=np.float32)
            check(L.pa_result_values(self._res.ptr, self._lane, _fp(out)))
            return out
        return self._get("values", f)

    @property
    def traceback_has_max_degree_1(self):
        return bool(lib().pa_result_max_degree_1(self._res.ptr))

    @property
    def traceback_as_matrix(self):
        def f():
            L = lib()
            k = L.pa_result_layers(self._res.ptr, self._lane)
            out = np.zeros((k, self._ls + 1, self._lt + 1, 2), dtype=np.int32)
            check(L.pa_result_tb_matrix(self._res.ptr, self._lane, _ip(out)))
            return _narrow(out, self._dtype)
        return self._get("tbm", f)

    @property
    def traceback_as_edges(self):
        def f():
            L = lib()
            k = L.pa_result_layers(self._res.ptr, self._lane)
            out = []
            for layer in range(k):
                n = L.pa_result_tb_edges(self._res.ptr, self._lane, layer, None)
                e = np.zeros((n, 2, 2), dtype=np.int32)
                if n:
                    L.pa_result_tb_edges(self._res.ptr, self._lane, layer, _ip(e))
                out.append(_narrow(e, self._dtype))
            return out
        return list(self._get("edges", f))

    def _walk(self):
        def f():
            if self._step is not None:
                return self._step
            L = lib()
            if not L.pa_result_has_alignment(self._res.ptr, self._lane):
                return None
            if self._first is not None:
                # the first result of the lane's search, from one device enumeration of
                # every lane of the result
                fa = self._first()
                if fa.counts[self._lane] > 0:
                    mp, path = fa.alignment(self._lane, 0)
                    return (float(L.pa_result_score(self._res.ptr, self._lane)), mp.copy(), path.copy())
            path = np.zeros((self._ls + self._lt + 4, 2), dtype=np.int32)
            n = L.pa_result_path(self._res.ptr, self._lane, _ip(path))
            mp = np.zeros((min(self._ls, self._lt),), dtype=np.int32)
            L.pa_result_alignment(self._res.ptr, self._lane, _ip(mp))
            sc = L.pa_result_score(self._res.ptr, self._lane)
            return (float(sc), mp, path[:max(n, 0)].copy() if n >= 0 else None)
        return self._get("walk", f)

    @property
    def path(self):
        w = self._walk()
        if w is None or w[2] is None:
            return None
        return _narrow(w[2], self._dtype)

    @property
    def score(self):
        w = self._walk()
        return None if w is None else float(w[0])

    @property
    def alignment(self):
        w = self._walk()
        if w is None:
            return None
        return Alignment(self._ls, self._lt, w[0], w[1], self._dtype)

    @property
    def algorithm(self):
        if not self._with_algorithm:
            return None
        L = lib()
        return Algorithm(*(L.pa_result_algorithm(self._res.ptr, k).decode() for k in range(3)))


class FirstAlignments:
    """The first k optimal alignments of every lane of an all-optimal result, enumerated on
    the GPU in one pass (pa_result_first_alignments): what the first k next() calls of each
    lane's iterator return.  `counts[lane]` results per lane (fewer than k: the lane has no
    more); `alignment(lane, j)` -> the j-th map (s_to_t if |s| <= |t|, else t_to_s) and, when
    enumerated with paths, the j-th walk ((n, 2) points)."""

    __slots__ = ("k", "counts", "maps", "mstart", "msize", "paths", "plen", "pstart", "pstride")

    def __init__(self, res, k, with_paths=False):
        L = lib()
        n = L.pa_result_size(res.ptr)
        ls = np.zeros(n, np.int32)
        lt = np.zeros(n, np.int32)
        check(L.pa_result_lengths(res.ptr, _ip(ls), _ip(lt)))
        self.k = int(k)
        self.msize = np.minimum(ls, lt).astype(np.int64)
        self.mstart = np.zeros(n, np.int64)
        self.mstart[1:] = np.cumsum(self.msize)[:-1] * self.k
        self.counts = np.zeros(n, np.int32)
        self.maps = np.zeros(max(1, int(self.msize.sum()) * self.k), np.int32)
        self.paths = self.plen = self.pstart = self.pstride = None
        if with_paths:
            self.pstride = (ls.astype(np.int64) + lt + 2)
            self.pstart = np.zeros(n, np.int64)
            self.pstart[1:] = np.cumsum(self.pstride)[:-1] * self.k
            self.paths = np.zeros((max(1, int(self.pstride.sum()) * self.k), 2), np.int32)
            self.plen = np.zeros(n * self.k, np.int32)
        st = L.pa_result_first_alignments(res.ptr, self.k, _ip(self.counts), _ip(self.maps),
                                          _ip(self.paths) if with_paths else None,
                                          _ip(self.plen) if with_paths else None)
        if st == PA_ERR_UNSUPPORTED:
            raise NotImplementedError(L.pa_last_error().decode())
        check(st)

    def alignment(self, lane, j):
        m = int(self.msize[lane])
        a = int(self.mstart[lane]) + j * m
        path = None
        if self.paths is not None:
            b = int(self.pstart[lane]) + j * int(self.pstride[lane])
            path = self.paths[b:b + int(self.plen[lane * self.k + j])]
        return self.maps[a:a + m], path


_ENUM_BYTES = 1 << 30  # host memory the iterators' device enumeration may fill


def _enumerated(res, with_paths):
    """The device enumeration backing a result's all-optimal iterators, made at the first
    next() of any of its lanes: the first k results of every lane, k = 101 (one more than
    pyalign's List codomain takes, so its exhaustion test is served too; PA_ENUM_FIRST sets k,
    0 turns this off), lowered so the results fit _ENUM_BYTES.  None when the result is not an
    all-optimal one with linear or affine gaps (its iterators run on the host)."""
    key = bool(with_paths)
    if key in res._first:
        return res._first[key]
    k = int(os.environ.get("PA_ENUM_FIRST", "101"))
    f = None
    if k > 0:
        L = lib()
        n = L.pa_result_size(res.ptr)
        ls = np.zeros(n, np.int32)
        lt = np.zeros(n, np.int32)
        check(L.pa_result_lengths(res.ptr, _ip(ls), _ip(lt)))
        per = 4 * int(np.minimum(ls, lt).sum()) + 12 * n
        if with_paths:
            per += 8 * int((ls.astype(np.int64) + lt + 2).sum()) + 4 * n
        k = min(k, _ENUM_BYTES // max(per, 1))
        if k > 0:
            try:
                f = FirstAlignments(res, k, with_paths)
            except NotImplementedError:
                f = None
    res._first[key] = f
    return f


class _Iter:
    _with_paths = False

    def __init__(self, res, lane, ls, lt, dtype):
        self._res, self._lane, self._ls, self._lt, self._dtype = res, lane, ls, lt, dtype
        self._it = None      # the host search, made when the device results run out
        self._served = 0     # results returned so far

    def __del__(self):
        if getattr(self, "_it", None) and _lib is not None:
            _lib.pa_iterator_destroy(self._it)
            self._it = None

    def path_count(self):
        """Number of co-optimal traceback paths of this lane -- the number of results this
        iterator yields when the solver's options keep duplicates (return_dup), computed on
        the GPU for every lane of the solve at once (pa_result_path_counts); uint64,
        saturating at 2**64 - 1.  All-optimal results with linear or affine gaps only."""
        return int(path_counts(self._res)[self._lane])

    def _next(self):
        L = lib()
        f = _enumerated(self._res, self._with_paths)
        if f is not None:
            c = int(f.counts[self._lane])
            if self._served < c:
                mp, path = f.alignment(self._lane, self._served)
                self._served += 1
                return float(L.pa_result_score(self._res.ptr, self._lane)), mp.copy(), \
                    (path.copy() if path is not None else np.zeros((0, 2), np.int32))
            if c < f.k:
                return None
        if self._it is None:
            # the host search (pa_iterator_next), resumed after the results already served
            h = _P()
            check(L.pa_result_iterator(self._res.ptr, self._lane, ctypes.byref(h)))
            self._it = h
            for _ in range(self._served):
                if not L.pa_iterator_next(h, None, None, None, None):
                    return None
        sc = ctypes.c_float(0)
        mp = np.zeros((min(self._ls, self._lt),), dtype=np.int32)
        path = np.zeros((self._ls + self._lt + 4, 2), dtype=np.int32)
        n = ctypes.c_int64(0)
        if not L.pa_iterator_next(self._it, ctypes.byref(sc), _ip(mp), _ip(path), ctypes.byref(n)):
            return None
        self._served += 1
        return float(sc.value), mp, path[:n.value].copy()


def path_counts(res):
    """Co-optimal traceback path count per lane of an all-optimal result (uint64 array)."""
    cached = res._path_counts
    if cached is None:
        cached = np.zeros(lib().pa_result_size(res.ptr), dtype=np.uint64)
        check(lib().pa_result_path_counts(res.ptr, cached.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        res._path_counts = cached
    return cached


class AlignmentIterator(_Iter):
    """AlignmentIterator (factory.h:218-245): next() -> Alignment or None."""

    def next(self):
        r = self._next()
        if r is None:
            return None
        return Alignment(self._ls, self._lt, r[0], r[1], self._dtype)


class SolutionIterator(_Iter):
    """SolutionIterator (factory.h:271-385): next() -> Solution or None."""

    _with_paths = True

    def next(self):
        r = self._next()
        if r is None:
            return None
        return Solution(self._res, self._lane, self._ls, self._lt, self._dtype, step=r, algorithm=False)


# --- solver ---

class Solver:
    """Solver (factory.h:414-508) running on the GPU."""

    def __init__(self, max_len_s, max_len_t, options):
        o = options
        self._opts = o
        self._index_dtype = np.int16 if o.index_bits == 16 else np.int32
        c = _Options()
        c.type, c.direction = int(o.type), int(o.direction)
        c.detail, c.count, c.locality = int(o.detail), int(o.count), int(o.locality)
        c.remove_dup, c.batch, c.batch_size = int(o.remove_dup), int(o.batch), int(o.batch_size)
        c.index_bits = int(o.index_bits)
        kinds = (o.gap_s[0], o.gap_t[0])
        self._keep = []
        if o.type == Type.DTW or kinds == ("linear", "linear"):
            c.gap_kind = 0
            c.linear_s, c.linear_t = float(o.gap_s[1]), float(o.gap_t[1])
        elif kinds == ("affine", "affine"):
            c.gap_kind = 1
            c.affine_u_s, c.affine_v_s = float(o.gap_s[1][0]), float(o.gap_s[1][1])
            c.affine_u_t, c.affine_v_t = float(o.gap_t[1][0]), float(o.gap_t[1][1])
        else:
            c.gap_kind = 2
            gs = _general_costs(o.gap_s, int(max_len_s) + 1)
            gt = _general_costs(o.gap_t, int(max_len_t) + 1)
            self._keep += [gs, gt]
            c.general_s, c.general_t = _fp(gs), _fp(gt)
        h = _P()
        check(lib().pa_solver_create(ctypes.byref(c), int(max_len_s), int(max_len_t), ctypes.byref(h)))
        self._h = h
        self._batch_size = lib().pa_solver_batch_size(h)
        # all-optimal iterators with linear or affine gaps enumerate on the device
        self._enumerable = o.type != Type.DTW and int(o.count) == int(Count.ALL) and c.gap_kind != 2
        # one-optimal alignments with linear, affine or DTW costs: maps straight into the
        # call's array (pa_solve_batch_result)
        self._direct_maps = o.type == Type.DTW or (int(o.count) == int(Count.ONE) and
                                                   int(o.detail) != int(Detail.SCORE) and c.gap_kind != 2)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.pa_solver_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def options(self):
        return self._opts.to_dict()

    @property
    def batch_size(self):
        return self._batch_size

    def last_timings(self):
        ms = (ctypes.c_float * 4)()
        n = ctypes.c_int32(0)
        lib().pa_solver_last_timings(self._h, ms, ctypes.byref(n))
        return list(ms), n.value

    KERNELS = ("one-column", "two-column", "stripe-chained", "16-bit twins", "general gaps", "16-bit twins, two-column",
               "16-bit twins, 4x4 blocks")

    def last_plan(self):
        """(kernel family, lanes per pair group, arithmetic, graph replay) of the last solve, and
        the group width per length bucket of |s| (<= 128, <= 256, <= 512, longer) when the
        launch gave each bucket its own (else None)."""
        v = (ctypes.c_int32 * 4)()
        lib().pa_solver_last_plan(self._h, v)
        w = (ctypes.c_int32 * 4)()
        lib().pa_solver_last_bucket_widths(self._h, w)
        return {"kernel": self.KERNELS[v[0]], "G": v[1], "arithmetic": ("float32", "int32", "int16x2")[v[2]],
                "graph": bool(v[3]), "bucket_widths": list(w) if any(w) else None}

    # --- argument marshalling (pytensor casts of factory.h:424-507)
    @staticmethod
    def _len(length):
        return np.ascontiguousarray(length, dtype=np.int32)

    @staticmethod
    def _codes(x):
        return np.ascontiguousarray(x, dtype=np.uint32)

    def _inputs(self, form, args):
        """Checked and converted arguments of a solve call (factory.h:424-507): the C
        arguments before the outputs, the arrays they point into, and a pa_batch of them."""
        def batch_check(given):  # factory.h:387-394, checked before the lengths (526-533)
            if given != self._batch_size:
                raise ValueError(f"problem of batch size {given} given to solver that was "
                                 f"configured to batch size {self._batch_size}")

        if form == "dense":
            sim, length = args
            sim = np.ascontiguousarray(sim, dtype=np.float32)
            if sim.ndim != 3:
                raise ValueError("similarity must be a 3-d array (len_s, len_t, batch)")
            batch_check(sim.shape[2])
            ln = self._len(length)
            head = [self._h, _fp(sim), sim.shape[0], sim.shape[1], sim.shape[2], _ip(ln)]
            keep = (sim, ln)
            lens = ln
        elif form == "indexed":
            a, b, sim, length = args
            a, b = self._codes(a), self._codes(b)
            sim = np.ascontiguousarray(sim, dtype=np.float32)
            batch_check(a.shape[0])
            batch_check(b.shape[0])
            ln = self._len(length)
            head = [self._h, _up(a), _up(b), a.shape[0], a.shape[1], b.shape[1], _fp(sim),
                    sim.shape[0], sim.shape[1], _ip(ln)]
            keep = (a, b, sim, ln)
            lens = ln
        else:
            a, b, eq, ne, length = args
            a, b = self._codes(a), self._codes(b)
            batch_check(a.shape[0])
            batch_check(b.shape[0])
            ln = self._len(length)
            head = [self._h, _up(a), _up(b), a.shape[0], a.shape[1], b.shape[1], float(eq), float(ne), _ip(ln)]
            keep = (a, b, ln)
            lens = ln
        if lens.ndim != 2 or lens.shape[0] != 2 or lens.shape[1] != self._batch_size:
            raise ValueError(f"m_length has shape {tuple(lens.shape)}, expected (2, {self._batch_size})")
        if form == "dense":
            bt = Batch(form=0, location=0, batch=sim.shape[2], n_s=sim.shape[0], n_t=sim.shape[1], sim=_fp(sim),
                       length=_ip(ln))
        elif form == "indexed":
            bt = Batch(form=1, location=0, batch=a.shape[0], n_s=a.shape[1], n_t=b.shape[1], a=_up(a), b=_up(b),
                       table=_fp(sim), table_rows=sim.shape[0], table_cols=sim.shape[1], length=_ip(ln))
        else:
            bt = Batch(form=2, location=0, batch=a.shape[0], n_s=a.shape[1], n_t=b.shape[1], a=_up(a), b=_up(b),
                       eq=float(eq), ne=float(ne), length=_ip(ln))
        return head, keep, bt

    def _call(self, name, form, args):
        L = lib()
        head, keep, _ = self._inputs(form, args)
        prefix = {"dense": "pa_solve_for_", "indexed": "pa_solve_indexed_for_", "binary": "pa_solve_binary_for_"}[form]
        fn = getattr(L, prefix + name)
        if name == "score":
            out = np.zeros((self._batch_size,), dtype=np.float32)
            check(fn(*head, _fp(out)))
            del keep
            return out
        h = _P()
        check(fn(*head, ctypes.byref(h)))
        del keep
        return _Result(h)

    def _lanes(self, res):
        L = lib()
        n = L.pa_result_size(res.ptr)
        ls = np.zeros((n,), dtype=np.int32)
        lt = np.zeros((n,), dtype=np.int32)
        if n:
            check(L.pa_result_lengths(res.ptr, _ip(ls), _ip(lt)))
        return n, ls.tolist(), lt.tolist()

    def _alignments(self, res):
        n, ls, lt = self._lanes(res)
        sizes = np.minimum(np.asarray(ls, dtype=np.int64), np.asarray(lt, dtype=np.int64))
        offs = np.zeros((n,), dtype=np.int64)
        if n > 1:
            offs[1:] = np.cumsum(sizes)[:-1]
        scores = np.zeros((n,), dtype=np.float32)
        if self._enumerable and n:
            # all-optimal solver: each lane's alignment is the first result of the depth-first
            # search (solver.h:2610-2630), enumerated for every lane at once on the device
            maps = FirstAlignments(res, 1).maps
            check(lib().pa_result_export(res.ptr, _fp(scores), None, None))
        else:
            maps = np.zeros((int(sizes.sum()),), dtype=np.int32)
            check(lib().pa_result_export(res.ptr, _fp(scores), _ip(maps), offs.ctypes.data_as(_PL)))
        batch = _AlignmentBatch(scores, maps, offs, sizes, ls, lt, self._index_dtype)
        return _Lanes(functools.partial(Alignment._lazy, batch), n)

    def _iterators(self, res, cls):
        n, ls, lt = self._lanes(res)
        if not self._enumerable:
            res._first = {False: None, True: None}  # one-optimal or general gaps: host iterators
        dt = self._index_dtype
        return _Lanes(lambda k: cls(res, k, ls[k], lt[k], dt), n)

    def _solutions(self, res):
        n, ls, lt = self._lanes(res)
        dt = self._index_dtype
        first = None
        if self._enumerable:
            def first():
                f = res._first.get("solution")
                if f is None:
                    f = res._first["solution"] = FirstAlignments(res, 1, with_paths=True)
                return f
        return _Lanes(lambda k: Solution(res, k, ls[k], lt[k], dt, first=first), n)

    def _alignment_call(self, form, args):
        """solve_*_for_alignment: the maps go straight into this call's array
        (pa_solve_batch_result), the scores come from the result object."""
        L = lib()
        head, keep, bt = self._inputs(form, args)
        n = int(bt.batch)
        ln = keep[-1]
        ls = np.clip(ln[0], 0, int(bt.n_s)).astype(np.int64)  # the lengths as the solve clamps them
        lt = np.clip(ln[1], 0, int(bt.n_t)).astype(np.int64)
        sizes = np.minimum(ls, lt)
        offs = np.zeros((n,), dtype=np.int64)
        if n > 1:
            np.cumsum(sizes[:-1], out=offs[1:])
        maps = np.empty((int(sizes.sum()),), dtype=np.int32)
        h = _P()
        check(L.pa_solve_batch_result(self._h, ctypes.byref(bt), _ip(maps), offs.ctypes.data_as(_PL), ctypes.byref(h)))
        del keep
        res = _Result(h)
        scores = np.empty((n,), dtype=np.float32)
        check(L.pa_result_export(res.ptr, _fp(scores), None, None))
        batch = _AlignmentBatch(scores, maps, offs, sizes, ls, lt, self._index_dtype)
        return _Lanes(functools.partial(Alignment._lazy, batch), n)

    def _dispatch(self, codomain, form, args):
        if codomain == "score":
            return self._call("score", form, args)
        if codomain == "alignment" and self._direct_maps:
            return self._alignment_call(form, args)
        res = self._call(codomain, form, args)
        if codomain == "alignment":
            return self._alignments(res)
        if codomain == "alignment_iterator":
            return self._iterators(res, AlignmentIterator)
        if codomain == "solution":
            return self._solutions(res)
        return self._iterators(res, SolutionIterator)

    def solve_for_score(self, sim, length):
        return self._dispatch("score", "dense", (sim, length))

    def solve_indexed_for_score(self, a, b, sim, length):
        return self._dispatch("score", "indexed", (a, b, sim, length))

    def solve_binary_for_score(self, a, b, eq, ne, length):
        return self._dispatch("score", "binary", (a, b, eq, ne, length))

    def solve_for_alignment(self, sim, length):
        return self._dispatch("alignment", "dense", (sim, length))

    def solve_for_alignment_iterator(self, sim, length):
        return self._dispatch("alignment_iterator", "dense", (sim, length))

    def solve_indexed_for_alignment(self, a, b, sim, length):
        return self._dispatch("alignment", "indexed", (a, b, sim, length))

    def solve_indexed_for_alignment_iterator(self, a, b, sim, length):
        return self._dispatch("alignment_iterator", "indexed", (a, b, sim, length))

    def solve_binary_for_alignment(self, a, b, eq, ne, length):
        return self._dispatch("alignment", "binary", (a, b, eq, ne, length))

    def solve_binary_for_alignment_iterator(self, a, b, eq, ne, length):
        return self._dispatch("alignment_iterator", "binary", (a, b, eq, ne, length))

    def solve_for_solution(self, sim, length):
        return self._dispatch("solution", "dense", (sim, length))

    def solve_for_solution_iterator(self, sim, length):
        return self._dispatch("solution_iterator", "dense", (sim, length))

    def solve_indexed_for_solution(self, a, b, sim, length):
        return self._dispatch("solution", "indexed", (a, b, sim, length))

    def solve_indexed_for_solution_iterator(self, a, b, sim, length):
        return self._dispatch("solution_iterator", "indexed", (a, b, sim, length))

    def solve_binary_for_solution(self, a, b, eq, ne, length):
        return self._dispatch("solution", "binary", (a, b, eq, ne, length))

    def solve_binary_for_solution_iterator(self, a, b, eq, ne, length):
        return self._dispatch("solution_iterator", "binary", (a, b, eq, ne, length))


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
        return Options(d, self._bits)

    def create_solver(self, max_len_s, max_len_t, options):
        return Solver(max_len_s, max_len_t, options)


m16 = _IndexModule(16)
m32 = _IndexModule(32)
