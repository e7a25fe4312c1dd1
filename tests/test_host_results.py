"""Host-side result objects and bag grouping of the native module (CPU only, no solve).

A solve call returns its per-lane results as a lazily filled sequence (`_Lanes`) of lazy
`Alignment` objects that read one exported batch (`_AlignmentBatch`); pyalign's Python
layer consumes that sequence like the tuple the reference's methods return
(factory.h:699-808) and reads `score`, `s_to_t` and `t_to_s` of each entry
(factory.h:130-193: the shorter side's map is stored, the other one is its inverse, -1
where unaligned).  `prepare.bag_batches` replaces `ProblemBag.batches`
(instance.py:230-275): every problem in exactly one batch, each batch's master shape
covering its members.  Options map pyalign's gap costs to the native special cases
(factory.h:33-90: affine (u, v) flipped to Gotoh's form, linear, none, general vectors,
per-side dicts).  These checks need no device: they build the exported arrays and the
gap objects by hand.
"""

import sys
import types

import numpy as np
import pytest

from pyalign_gb300 import algorithm as alg
from pyalign_gb300 import prepare


def _brute_inverse(mp, n):
    out = np.full(n, -1, dtype=np.int64)
    for i, j in enumerate(mp):
        if j >= 0:
            out[j] = i
    return out


def test_lanes_behave_like_a_tuple_and_make_each_entry_once():
    made = []

    def make(k):
        made.append(k)
        return ("lane", k)

    seq = alg._Lanes(make, 5)
    assert len(seq) == 5 and made == []           # nothing made by the call itself
    assert seq[3] == ("lane", 3) and seq[-1] == ("lane", 4)
    assert seq[3] is seq[3] and made == [3, 4]    # made once, kept
    assert seq[1:4] == (("lane", 1), ("lane", 2), ("lane", 3))
    assert isinstance(seq[::-2], tuple) and seq[::-2] == (("lane", 4), ("lane", 2), ("lane", 0))
    assert list(seq) == [("lane", k) for k in range(5)]
    assert sorted(made) == [0, 1, 2, 3, 4]        # every entry made exactly once
    a, *rest = seq
    assert a == ("lane", 0) and len(rest) == 4
    assert list(zip(range(2), seq)) == [(0, ("lane", 0)), (1, ("lane", 1))]
    for bad in (5, -6):
        with pytest.raises(IndexError):
            seq[bad]
    with pytest.raises(TypeError):
        seq[1.0]
    assert len(alg._Lanes(make, 0)) == 0 and list(alg._Lanes(make, 0)) == []


@pytest.mark.parametrize("dtype", [np.int16, np.int32])
def test_lazy_alignments_read_their_lane_of_the_batch(dtype):
    rng = np.random.default_rng(5)
    ls = [0, 7, 12, 5, 9, 1]
    lt = [4, 7, 5, 11, 9, 0]
    sizes = np.minimum(ls, lt).astype(np.int64)
    offs = np.zeros(len(ls), dtype=np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    maps = np.full(int(sizes.sum()), -1, dtype=np.int32)
    want = []
    for k, (s, t) in enumerate(zip(ls, lt)):
        m, n = min(s, t), max(s, t)
        # an increasing partial map of the shorter side into the longer one
        cols = np.sort(rng.choice(n, size=m, replace=False)) if m else np.zeros(0, np.int64)
        keep = rng.random(m) < 0.7
        mp = np.where(keep, cols, -1)
        maps[offs[k]:offs[k] + m] = mp
        want.append(mp)
    scores = rng.normal(size=len(ls)).astype(np.float32)
    batch = alg._AlignmentBatch(scores, maps, offs, sizes, ls, lt, dtype)
    seq = alg._Lanes(lambda k: alg.Alignment._lazy(batch, k), len(ls))
    for k, a in enumerate(seq):
        s, t = ls[k], lt[k]
        assert a.score == float(scores[k])
        short = a.s_to_t if s <= t else a.t_to_s
        other = a.t_to_s if s <= t else a.s_to_t
        assert short.dtype == dtype and other.dtype == dtype
        assert short.shape == (min(s, t),) and other.shape == (max(s, t),)
        np.testing.assert_array_equal(short, want[k])
        np.testing.assert_array_equal(other, _brute_inverse(want[k], max(s, t)))
        # an eagerly built Alignment of the same lane is the same object to a reader
        e = alg.Alignment(s, t, scores[k], want[k].astype(np.int32), dtype)
        assert e.score == a.score
        np.testing.assert_array_equal(e.s_to_t, a.s_to_t)
        np.testing.assert_array_equal(e.t_to_s, a.t_to_s)


def test_narrowing_keeps_minus_one_and_maps_the_none_marker():
    none32 = np.iinfo(np.int32).min
    a = np.array([-1, 0, 5, 32767, none32], dtype=np.int32)
    n16 = alg._narrow(a, np.int16)
    assert n16.dtype == np.int16
    assert n16.tolist() == [-1, 0, 5, 32767, np.iinfo(np.int16).min]
    n32 = alg._narrow(a, np.int32)
    assert n32.dtype == np.int32 and n32.tolist() == a.tolist()


@pytest.fixture
def fake_instance(monkeypatch):
    """pyalign.problems.instance with just its ProblemBatch record (instance.py:168-186)."""
    class ProblemBatch:
        def __init__(self, problems, indices, master_shape):
            self.problems, self.indices, self.shape = problems, indices, master_shape

    mod = types.ModuleType("pyalign.problems.instance")
    mod.ProblemBatch = ProblemBatch
    pkg = types.ModuleType("pyalign")
    sub = types.ModuleType("pyalign.problems")
    pkg.problems, sub.instance = sub, mod
    for name, m in (("pyalign", pkg), ("pyalign.problems", sub), ("pyalign.problems.instance", mod)):
        monkeypatch.setitem(sys.modules, name, m)
    return mod


@pytest.mark.parametrize("batch_size", [1, 3, 64, 1000])
def test_bag_batches_cover_every_problem_once(fake_instance, batch_size):
    rng = np.random.default_rng(batch_size)
    shapes = [(int(rng.integers(0, 50)), int(rng.integers(0, 50))) for _ in range(257)]
    shapes += [(7, 7)] * 5                                    # equal shapes
    problems = [types.SimpleNamespace(shape=s, tag=k) for k, s in enumerate(shapes)]
    bag = types.SimpleNamespace(problems=problems)
    seen = []
    for batch in prepare.bag_batches(bag, batch_size):
        assert isinstance(batch, fake_instance.ProblemBatch)
        assert 1 <= len(batch.indices) <= batch_size
        assert [p.tag for p in batch.problems] == list(batch.indices)
        ms, mt = batch.shape
        assert all(problems[i].shape[0] <= ms and problems[i].shape[1] <= mt for i in batch.indices)
        assert (ms, mt) == (max(problems[i].shape[0] for i in batch.indices),
                            max(problems[i].shape[1] for i in batch.indices))
        seen.extend(batch.indices)
    assert sorted(seen) == list(range(len(problems)))
    assert list(prepare.bag_batches(types.SimpleNamespace(problems=[]), batch_size)) == []


class _Gap:
    """A gap cost as pyalign.gaps presents it to the native module: to_special_case() and
    costs(n) (gaps.py:13-17)."""

    def __init__(self, special, costs=None):
        self._special, self._costs = special, costs

    def to_special_case(self):
        return dict(self._special)

    def costs(self, n):
        return self._costs(n)


def _options(gap_cost, **extra):
    d = {"solver": alg.Type.ALIGNMENT, "direction": alg.Direction.MAXIMIZE, "batch": True,
         "return_dup": False, "locality": alg.Locality.GLOBAL, "gap_cost": gap_cost,
         "codomain": types.SimpleNamespace(detail=alg.Detail.ALIGNMENT, count=alg.Count.ONE)}
    d.update(extra)
    return alg.m16.create_options(d)


def test_gap_costs_map_to_the_native_special_cases():
    # affine (u, v) of w(k) = u + v k becomes Gotoh's (u', v') = (v, u) (factory.h:42-52)
    o = _options(_Gap({"affine": (3.0, 2.0)}))
    assert o.gap_s == o.gap_t
    kind, (ext, opn) = o.gap_s
    assert kind == "affine" and (float(ext), float(opn)) == (2.0, 3.0)
    w = alg._general_costs(o.gap_s, 6)
    assert w.dtype == np.float32 and w.tolist() == [0.0, 5.0, 7.0, 9.0, 11.0, 13.0]
    # linear, and no gap cost at all (linear 0, factory.h:37-38)
    o = _options(_Gap({"linear": 1.5}))
    assert o.gap_s[0] == "linear" and float(o.gap_s[1]) == 1.5
    assert alg._general_costs(o.gap_s, 4).tolist() == [0.0, 1.5, 3.0, 4.5]
    o = _options(None)
    assert o.gap_s[0] == "linear" and float(o.gap_s[1]) == 0.0
    # a gap cost with no special case is general: its cost vector, length-checked
    g = _Gap({}, lambda n: np.log(np.arange(n, dtype=np.float64) + 1.0))
    o = _options(g)
    assert o.gap_s == ("general", g)
    np.testing.assert_array_equal(alg._general_costs(o.gap_s, 5), np.log(np.arange(5) + 1.0).astype(np.float32))
    with pytest.raises(ValueError):
        alg._general_costs(("general", _Gap({}, lambda n: np.zeros(n + 1))), 5)


def test_per_side_gap_costs_and_option_defaults():
    # a dict gives each side its own cost; a missing side has none (factory.h:70-86)
    o = _options({"s": _Gap({"linear": 2.0}), "t": _Gap({"affine": (1.0, 0.5)})})
    assert o.gap_s[0] == "linear" and float(o.gap_s[1]) == 2.0
    assert o.gap_t[0] == "affine" and tuple(map(float, o.gap_t[1])) == (0.5, 1.0)
    o = _options({"t": _Gap({"linear": 2.0})})
    assert o.gap_s[0] == "linear" and float(o.gap_s[1]) == 0.0
    assert o.remove_dup and o.locality == alg.Locality.GLOBAL and o.index_bits == 16
    o = _options(None, return_dup=True, batch_size=77)
    assert not o.remove_dup and o.batch_size == 77
    d = _options(None).to_dict()
    del d["locality"]
    assert alg.m32.create_options(d).locality == alg.Locality.LOCAL
    assert alg.m32.create_options(d).index_bits == 32
    # DTW options carry no gap costs and are global, one optimum
    dtw = alg.m16.create_options({"solver": alg.Type.DTW, "direction": alg.Direction.MINIMIZE,
                                  "batch": True, "return_dup": False})
    assert dtw.locality == alg.Locality.GLOBAL and dtw.count == alg.Count.ONE
    # illegal enum values are refused, as pybind11 refuses them
    with pytest.raises(ValueError):
        _options(None, direction=7)
