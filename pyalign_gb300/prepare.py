"""Batch problem preparation: one call encodes every sequence of a batch.

pyalign's indexed form prepares a batch problem by problem (pyalign/solve.py:382-396:
``p.build_index_sequences(a[k, :shape[0]], b[k, :shape[1]])`` for each problem), and an
alphabet problem encodes each of its strings on its own (pyalign/problems/factory.py:87-90,
``ByteAlphabetEncoder.encode``, factory.py:114-127: latin1 bytes mapped through a 256-entry
index, 0xff = not in the alphabet -> ``ValueError("item not in alphabet")``).  With
thousands of pairs per batch that Python loop costs more than the solve.  Here the strings
of a whole batch are joined into one byte buffer and encoded by one C-ABI call
(``pa_encode_latin1``): into host arrays by worker threads, or into device arrays from a
single upload of the raw bytes.

``patch_prepare()`` installs the batch encoder as the indexed form's ``prepare`` for
batches of byte-alphabet problems (all sharing one ``ByteAlphabetEncoder``); other batches
keep pyalign's own method.  The codes written are the ones the per-problem encoder writes
(it uses the encoder's own index table), so the solve is unchanged; rows are zero-padded
beyond each string where pyalign leaves earlier contents (never read: every cell beyond a
pair's lengths is outside its matrix).  One difference: an empty string, which the
reference's encoder rejects with numpy's zero-size reduction error, is accepted.
"""

import ctypes

import numpy as np

from . import algorithm as _alg

_P = ctypes.c_void_p


def _lib():
    L = _alg.lib()
    if not getattr(L, "_encode_declared", False):
        L.pa_encode_latin1.restype = ctypes.c_int32
        L.pa_encode_latin1.argtypes = [_P, _P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_int64, _P,
                                       ctypes.c_int32, _P]
        L._encode_declared = True
    return L


def lut_of(encoder):
    """The 256-entry byte -> code table of a ``ByteAlphabetEncoder`` (its ``_index``), or of
    an alphabet given as a string (code = position in the string)."""
    if isinstance(encoder, str):
        lut = np.full(256, 0xFF, np.uint8)
        for i, ch in enumerate(encoder):
            lut[ch.encode("latin1")[0]] = i
        return lut
    return np.ascontiguousarray(encoder._index, dtype=np.uint8)


def _join(strings):
    parts = [s if isinstance(s, str) else "".join(s) for s in strings]
    lens = np.fromiter((len(s) for s in parts), dtype=np.int64, count=len(parts))
    offsets = np.zeros(len(parts) + 1, np.int64)
    np.cumsum(lens, out=offsets[1:])
    return "".join(parts).encode("latin1"), offsets, lens


def encode_latin1(strings, lut, out=None, width=None, device=None, stream=None):
    """Encode ``strings`` (str or sequences of 1-character str) into the rows of ``out``:
    a (n, >= width) uint32 numpy array (host) or torch tensor on a CUDA device (int32 or
    uint32 view).  Without ``out`` a host array of width max(len) is returned.  ``lut`` is a
    256-entry uint8 table (``lut_of``).  Returns (codes, lengths)."""
    text, offsets, lens = _join(strings)
    n = len(lens)
    if width is None:
        width = int(lens.max()) if n else 0
    lut = np.ascontiguousarray(lut, dtype=np.uint8)
    if lut.shape != (256,):
        raise ValueError("lut must have 256 entries")
    if out is None:
        out = np.zeros((n, width), np.uint32)
    if isinstance(out, np.ndarray):
        if out.dtype != np.uint32 or out.ndim != 2 or out.shape[0] < n or out.shape[1] < width:
            raise ValueError("out must be a (n, >= width) uint32 array")
        if out.strides[1] != 4:
            raise ValueError("out rows must be contiguous")
        ptr, stride, loc = out.ctypes.data, out.strides[0] // 4, 0
    else:  # a CUDA tensor
        if out.dim() != 2 or out.element_size() != 4 or out.shape[0] < n or out.shape[1] < width or out.stride(1) != 1:
            raise ValueError("out must be a (n, >= width) 4-byte tensor with contiguous rows")
        ptr, stride, loc = out.data_ptr(), out.stride(0), 1
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(out.device).cuda_stream
    if device is not None and bool(device) != (loc == 1):
        raise ValueError("device= does not match where out lives")
    tp = ctypes.cast(ctypes.c_char_p(text), _P) if text else None  # the bytes object's own buffer
    _alg.check(_lib().pa_encode_latin1(tp, offsets.ctypes.data, n, lut.ctypes.data, width, stride, ptr, loc, stream))
    return out, lens


def _byte_alphabet_encoder(problems):
    """The ByteAlphabetEncoder shared by all problems of a batch, else None."""
    enc = getattr(problems[0], "_encoder", None) if problems else None
    if enc is None or type(enc).__name__ != "ByteAlphabetEncoder" or not hasattr(enc, "_index"):
        return None
    for p in problems:
        if getattr(p, "_encoder", None) is not enc or not hasattr(p, "_s") or not hasattr(p, "_t"):
            return None
    return enc


def batch_prepare(form, batch, original=None):
    """The indexed form's prepare (solve.py:382-396) for a batch of byte-alphabet problems:
    a[k, :|s_k|], b[k, :|t_k|] and the lengths of every problem k, in two encoder calls."""
    problems = batch.problems
    enc = _byte_alphabet_encoder(problems)
    if enc is None:
        if original is None:
            raise ValueError("batch_prepare needs byte-alphabet problems")
        return original(form, batch)
    shape = batch.shape
    lut = lut_of(enc)
    n = len(problems)
    encode_latin1([p._s for p in problems], lut, out=form._a[:n], width=shape[0])
    encode_latin1([p._t for p in problems], lut, out=form._b[:n], width=shape[1])
    for k, p in enumerate(problems):
        form._len[0, k], form._len[1, k] = p.shape
    return None


def patch_prepare(solve_module=None):
    """Install ``batch_prepare`` as ``AbstractIndexedMatrixForm.prepare`` of pyalign.solve
    (call after ``import pyalign``); returns the original method."""
    if solve_module is None:
        import pyalign.solve as solve_module
    cls = solve_module.AbstractIndexedMatrixForm
    original = cls.prepare
    if getattr(original, "_pa_batch_prepare", False):
        return original._pa_original

    def prepare(self, batch):
        return batch_prepare(self, batch, original)

    prepare._pa_batch_prepare = True
    prepare._pa_original = original
    cls.prepare = prepare
    return original


def bag_batches(bag, batch_size):
    """The batches of a ProblemBag for this library, in O(B log B): the problems sorted by
    shape (|s| then |t|, largest first) and cut into runs of ``batch_size``, each with its
    own largest shape as master shape.  pyalign's ProblemBag.batches (instance.py:230-275)
    groups by Morton order with a rescan of the remaining problems per batch, which at
    65,536 problems costs seconds of Python; the grouping only decides which lanes share a
    native call, and each lane's result depends on its own lengths alone, so any grouping
    whose master shape covers every member gives the same results.  Yields the same
    ProblemBatch objects (problems, indices, master_shape)."""
    from pyalign.problems.instance import ProblemBatch
    problems = bag.problems
    if batch_size == 1:
        for i, p in enumerate(problems):
            yield ProblemBatch([p], [i], p.shape)
        return
    shapes = np.array([p.shape for p in problems], dtype=np.int64).reshape(-1, 2)
    order = np.lexsort((-shapes[:, 1], -shapes[:, 0]))
    for k0 in range(0, len(order), batch_size):
        idx = order[k0:k0 + batch_size].tolist()
        master = (int(shapes[idx, 0].max()), int(shapes[idx, 1].max()))
        yield ProblemBatch([problems[i] for i in idx], idx, master)


def patch_batches(instance_module=None):
    """Install ``bag_batches`` as ``ProblemBag.batches`` of pyalign.problems.instance (call
    after ``import pyalign``; opt-in); returns the original method."""
    if instance_module is None:
        import pyalign.problems.instance as instance_module
    cls = instance_module.ProblemBag
    original = cls.batches
    if getattr(original, "_pa_bag_batches", False):
        return original._pa_original

    def batches(self, batch_size):
        return bag_batches(self, batch_size)

    batches._pa_bag_batches = True
    batches._pa_original = original
    cls.batches = batches
    return original
