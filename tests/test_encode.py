"""Batch encoding of byte-alphabet problems (CPU: the host path of pa_encode_latin1).

The reference encodes each string with ByteAlphabetEncoder.encode
(pyalign/problems/factory.py:114-127): latin1 bytes through a 256-entry index, 0xff -> 
ValueError("item not in alphabet"), written to out[:len].  Its indexed form prepares a batch
problem by problem (pyalign/solve.py:382-396).  Both are restated here on stand-ins with the
same attributes (the reference package is not importable), and the batch encoder and
batch_prepare must write the same codes and lengths.
"""

import numpy as np
import pytest

from pyalign_gb300 import prepare as prep


class ByteAlphabetEncoder:  # the attributes of factory.py:103-127 that the batch path reads
    def __init__(self, alphabet):
        self._alphabet = tuple(alphabet)
        self._index = np.full(256, 0xFF, np.uint8)
        for i, k in enumerate(self._alphabet):
            self._index[k.encode("latin1")[0]] = i

    def encode(self, s, out=None):
        if not isinstance(s, str):
            s = "".join(s)
        r = self._index[np.frombuffer(s.encode("latin1"), dtype=np.uint8)]
        if np.max(r) == 0xFF:
            raise ValueError("item not in alphabet")
        out[:len(r)] = r


class AlphabetProblem:
    def __init__(self, encoder, s, t):
        self._encoder, self._s, self._t = encoder, s, t
        self.shape = (len(s), len(t))

    def build_index_sequences(self, a, b):
        self._encoder.encode(self._s, out=a)
        self._encoder.encode(self._t, out=b)


class Batch:
    def __init__(self, problems):
        self.problems = problems
        self.shape = (max(p.shape[0] for p in problems), max(p.shape[1] for p in problems))


class Form:
    def __init__(self, batch_size, n_s, n_t):
        self._a = np.zeros((batch_size, n_s), np.uint32)
        self._b = np.zeros((batch_size, n_t), np.uint32)
        self._len = np.zeros((2, batch_size), np.uint16)


def reference_prepare(form, batch):  # solve.py:382-396
    shape = batch.shape
    for k, p in enumerate(batch.problems):
        p.build_index_sequences(form._a[k, :shape[0]], form._b[k, :shape[1]])
        form._len[0, k], form._len[1, k] = p.shape


def _strings(rng, n, alphabet, lo, hi):
    return ["".join(rng.choice(list(alphabet), size=int(rng.integers(lo, hi + 1)))) for _ in range(n)]


def test_host_encoding_matches_per_string_encoder():
    rng = np.random.default_rng(3)
    enc = ByteAlphabetEncoder("TGCA")
    strings = _strings(rng, 500, "ACGT", 1, 300)
    codes, lens = prep.encode_latin1(strings, prep.lut_of(enc))
    assert codes.shape == (500, max(len(s) for s in strings))
    for k, s in enumerate(strings):
        want = np.zeros(codes.shape[1], np.uint32)
        enc.encode(s, out=want)
        assert np.array_equal(codes[k], want), k
        assert lens[k] == len(s)


def test_sequences_of_letters_and_string_alphabets():
    codes, _ = prep.encode_latin1([list("GATTACA"), "CAT"], prep.lut_of("ACGT"), width=9)
    assert codes.tolist() == [[2, 0, 3, 3, 0, 1, 0, 0, 0], [1, 0, 3, 0, 0, 0, 0, 0, 0]]


def test_errors_match_reference():
    lut = prep.lut_of("ACGT")
    with pytest.raises(ValueError, match="item not in alphabet"):
        prep.encode_latin1(["ACGT", "ACGN"], lut)
    with pytest.raises(RuntimeError, match="longer"):
        prep.encode_latin1(["ACGTACGT"], lut, out=np.zeros((1, 8), np.uint32), width=4)


def test_batch_prepare_matches_reference_prepare():
    rng = np.random.default_rng(11)
    enc = ByteAlphabetEncoder("ACGT")
    problems = [AlphabetProblem(enc, s, t) for s, t in zip(_strings(rng, 300, "ACGT", 1, 200),
                                                            _strings(rng, 300, "ACGT", 1, 250))]
    batch = Batch(problems)
    want, got = Form(512, 200, 250), Form(512, 200, 250)
    reference_prepare(want, batch)
    prep.batch_prepare(got, batch)
    n_s, n_t = batch.shape
    assert np.array_equal(got._len, want._len)
    for k, p in enumerate(problems):  # the cells inside each pair's lengths
        assert np.array_equal(got._a[k, :p.shape[0]], want._a[k, :p.shape[0]])
        assert np.array_equal(got._b[k, :p.shape[1]], want._b[k, :p.shape[1]])
        assert not got._a[k, p.shape[0]:n_s].any() and not got._b[k, p.shape[1]:n_t].any()


def test_patch_prepare_dispatch():
    """The patched prepare encodes byte-alphabet batches and leaves other batches to the
    original method."""
    import types
    calls = []

    class AbstractIndexedMatrixForm:
        def prepare(self, batch):
            calls.append(batch)

    mod = types.SimpleNamespace(AbstractIndexedMatrixForm=AbstractIndexedMatrixForm)
    original = prep.patch_prepare(mod)
    assert prep.patch_prepare(mod) is original  # idempotent
    enc = ByteAlphabetEncoder("ACGT")
    form = Form(4, 8, 8)
    form.prepare = types.MethodType(AbstractIndexedMatrixForm.prepare, form)
    form.prepare(Batch([AlphabetProblem(enc, "ACG", "TTTT")]))
    assert not calls and form._a[0, :3].tolist() == [0, 1, 2] and form._len[:, 0].tolist() == [3, 4]

    class Other:
        _s, _t, shape = "AC", "GT", (2, 2)
    form.prepare(Batch([Other()]))
    assert len(calls) == 1
