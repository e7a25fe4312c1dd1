"""Differentiable optimal alignment scores (torch.autograd) on the GB300 kernels.

The reference has no gradients; this is the "differentiation" form of the batched solve.
The forward pass is the same sm_103a DP as the drop-in module (one optimal path per pair,
solver.h:2665-2705); the backward pass is the max-plus subgradient of the optimal score:
the indicator of the aligned cells of the optimal path for dScore/dS (every visited cell
for DTW) and the gap counts along the path for dScore/d(open, extend), computed by
`pa_path_gradients` from the paths the forward pass keeps on the device.  Gradients with
respect to embeddings flow through the similarity product by torch's autograd.

Tie-breaking follows the reference, so on inputs with ties the subgradient is the one of
the reference's optimal path.
"""

import ctypes
import types

import numpy as np
import torch

from . import algorithm as _alg

_SOLVERS = {}


class _Gap:
    def __init__(self, open_, extend):
        self.open, self.extend = float(open_), float(extend)

    def to_special_case(self):
        return {"affine": (self.open - self.extend, self.extend)}


class _Linear:
    def __init__(self, g):
        self.g = float(g)

    def to_special_case(self):
        return {"linear": self.g}


def _solver(batch, n_s, n_t, locality, direction, dtw, gap):
    key = (batch, n_s, n_t, locality, direction, dtw, gap)
    s = _SOLVERS.get(key)
    if s is None:
        A = _alg
        d = {
            "solver": A.Type.DTW if dtw else A.Type.ALIGNMENT,
            "direction": A.Direction.__members__[direction.upper()],
            "batch": True, "batch_size": batch, "return_dup": False,
            "locality": A.Locality.__members__[locality.upper()],
            "codomain": types.SimpleNamespace(detail=A.Detail.ALIGNMENT, count=A.Count.ONE),
            "gap_cost": None if dtw else (_Linear(gap[0]) if gap[1] is None else _Gap(*gap)),
        }
        mod = A.m32 if max(n_s, n_t) >= 16000 else A.m16
        s = mod.create_solver(n_s, n_t, mod.create_options(d))
        if len(_SOLVERS) > 32:
            _SOLVERS.clear()
        _SOLVERS[key] = s
    return s


def _lib():
    L = _alg.lib()
    if not getattr(L, "_pa_grad_bound", False):
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
        L.pa_solve_dense_paths.restype = i32
        L.pa_solve_dense_paths.argtypes = [vp, vp, vp, i64, i64, i64, i64, i64, vp, vp, vp, vp, vp]
        L.pa_solve_series_paths.restype = i32
        L.pa_solve_series_paths.argtypes = [vp, vp, i64, vp, i64, i64, i64, i64, vp, vp, vp, vp, vp]
        L.pa_path_gradients.restype = i32
        L.pa_path_gradients.argtypes = [i32, i32, i32, i64, vp, vp, vp, vp, vp, vp, i64, i64, vp, vp]
        L.pa_path_embedding_gradients.restype = i32
        L.pa_path_embedding_gradients.argtypes = [i64, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64, i64,
                                                  vp, vp, vp]
        L.pa_path_embedding_gradients_full.restype = i32
        L.pa_path_embedding_gradients_full.argtypes = L.pa_path_embedding_gradients.argtypes
        L.pa_normalize_rows_bf16.restype = i32
        L.pa_normalize_rows_bf16.argtypes = [vp, i64, i32, i32, vp, vp, vp]
        L.pa_normalize_rows_bf16_lengths.restype = i32
        L.pa_normalize_rows_bf16_lengths.argtypes = [vp, i64, i64, i32, i32, vp, vp, vp, vp]
        L.pa_normalize_rows_bf16_tiled.restype = i32
        L.pa_normalize_rows_bf16_tiled.argtypes = [vp, i64, i64, i32, i32, vp, i32, vp, vp, vp]
        L.pa_path_series_gradients.restype = i32
        L.pa_path_series_gradients.argtypes = [i64, vp, vp, vp, vp, vp, vp, i64, i64, vp, vp, vp]
        L.pa_similarity_bf16.restype = i32
        f32 = ctypes.c_float
        L.pa_similarity_bf16.argtypes = [vp, vp, i64, i64, i64, i32, vp, vp, vp, i64, vp, i64, i64, f32, f32, vp, vp]
        L.pa_path_scores_f64.restype = i32
        L.pa_path_scores_f64.argtypes = [i32, i32, i32, i64, vp, vp, vp, vp, vp, i64, i64, vp, vp, vp, vp]
        L._pa_grad_bound = True
    return L


_STATUS = {}


def _status(device):
    st = _STATUS.get(device)
    if st is None:
        st = torch.zeros(1, dtype=torch.int32, device=device)
        _STATUS[device] = st
    return st


def tensor_core_status(device=None):
    """Error bits the tensor-core similarity kernel raised since the last call (2: a wait
    for the tensor cores timed out); reading synchronises the device and clears them."""
    st = _status(torch.device(device or "cuda", torch.cuda.current_device()))
    v = int(st.item())
    st.zero_()
    return v


_small_cache = {}   # (device, dtype, bytes) -> device tensor: index arrays seen before
_staging = {}       # (device, dtype) -> (pinned buffer, event of its last copy)


def _to_device(arr, device):
    """A small host index array (lengths, offsets) on the device without blocking the host: a
    content-keyed cache (a training loop passes the same lengths every step) and, for new
    contents, a non-blocking copy out of a reused pinned buffer."""
    arr = np.ascontiguousarray(arr)
    device = torch.device(device)
    key = (str(device), arr.dtype.str, arr.shape, arr.tobytes())
    hit = _small_cache.get(key)
    if hit is not None:
        return hit
    dtype = torch.from_numpy(arr[:0]).dtype
    buf, ev = _staging.get((str(device), arr.dtype.str), (None, None))
    if buf is None or buf.numel() < arr.size:
        buf, ev = torch.empty(max(arr.size, 1 << 14), dtype=dtype, pin_memory=True), None
    if ev is not None:
        ev.synchronize()  # the previous copy out of the buffer has finished
    flat = buf[:arr.size]
    flat.copy_(torch.from_numpy(arr.reshape(-1)))
    out = flat.to(device, non_blocking=True).reshape(arr.shape)
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(device))
    _staging[(str(device), arr.dtype.str)] = (buf, ev)
    if len(_small_cache) >= 32:
        _small_cache.pop(next(iter(_small_cache)))
    _small_cache[key] = out
    return out


def _lengths(lengths, B):
    ln = np.ascontiguousarray(np.asarray(lengths).reshape(B, 2).T, dtype=np.int32)
    return ln


def similarity_bf16(Esb, Etb, lengths, out=None, alpha=1.0, beta=0.0):
    """S = beta + alpha <Es[i], Et[j]> per pair from BF16 factors (batch, n, dim), on the
    tensor cores (pa_similarity_bf16), FP32 accumulation (alpha = -1, beta = 1 gives the
    distance 1 - cos).  Only the cells inside each pair's lengths are written: the rest of
    `out` (a fresh torch.empty by default) is left as it was.  Returns S as a
    (batch, n_s, n_t) transposed view of S^T, stride 1 along s."""
    B, n_s, dim = Esb.shape
    n_t = Etb.shape[1]
    if Esb.dtype != torch.bfloat16 or Etb.dtype != torch.bfloat16 or not Esb.is_contiguous() \
            or not Etb.is_contiguous() or Etb.shape[0] != B or Etb.shape[2] != dim:
        raise ValueError("Es, Et must be contiguous BF16 (batch, n, dim) tensors of one batch and dim")
    if dim % 16:
        raise ValueError("dim must be a multiple of 16")
    ln = _lengths(lengths, B)
    if (ln[0] > n_s).any() or (ln[1] > n_t).any() or (ln < 0).any():
        raise ValueError("lengths exceed the embeddings")
    tiles = ((ln[1].astype(np.int64) + 127) // 128) * ((ln[0].astype(np.int64) + 127) // 128)
    meta = np.zeros(3 * B + 1, np.int32)
    meta[:B] = ln[0]
    meta[B:2 * B] = ln[1]
    meta[2 * B + 1:] = np.cumsum(tiles)
    total = int(meta[-1])
    dmeta = _to_device(meta, Esb.device)  # no host wait for the queued work
    if out is None:
        out = torch.empty((B, n_t, n_s), dtype=torch.float32, device=Esb.device)
    elif out.shape != (B, n_t, n_s) or out.dtype != torch.float32 or out.stride(2) != 1 or not out.is_cuda:
        raise ValueError("out must be a (batch, n_t, n_s) float32 CUDA tensor with unit stride along s")
    st = _status(Esb.device)
    _alg.check(_lib().pa_similarity_bf16(
        Esb.data_ptr(), Etb.data_ptr(), B, n_s, n_t, dim, dmeta.data_ptr(), dmeta.data_ptr() + 4 * B,
        dmeta.data_ptr() + 8 * B, total, out.data_ptr(), out.stride(0), out.stride(1), float(alpha), float(beta),
        st.data_ptr(),
        torch.cuda.current_stream().cuda_stream))
    return out.transpose(1, 2)


def _pad16(E):
    d = E.shape[-1]
    return E if d % 16 == 0 else torch.nn.functional.pad(E, (0, 16 - d % 16))


def path_scores_f64(S, lengths, gap_open=None, gap_extend=None, locality="global", direction="maximize",
                    dtw=False, with_scale=False):
    """The optimal scores of the float32 DP and, for the same recovered paths, their scores
    re-evaluated in FP64 on the GPU (pa_path_scores_f64): (scores float32, replay float64),
    plus with_scale the magnitude of the summed terms (sum |S| + gap costs) per path.  The
    distance between the two scores is the DP's float32 accumulation error."""
    linear = gap_extend is None
    gap = None if dtw else ((float(gap_open), None) if linear else (float(gap_open), float(gap_extend)))
    if S.stride(1) != 1 and S.stride(2) != 1:
        S = S.contiguous()
    scores, paths, plen, poff, _ = _forward_paths(S, lengths, gap, locality, direction, dtw)
    B = S.shape[0]
    A = _alg
    if dtw:
        g = None
    elif linear:
        g = np.array([gap[0], gap[0], gap[0], gap[0]], np.float64)
    else:
        g = np.array([gap[0], gap[1], gap[0], gap[1]], np.float64)
    soff = torch.from_numpy(S.storage_offset() + np.arange(B, dtype=np.int64) * S.stride(0)).to(S.device)
    base = S.data_ptr() - S.storage_offset() * S.element_size()
    out = torch.empty(B, dtype=torch.float64, device=S.device)
    scale = torch.empty(B, dtype=torch.float64, device=S.device) if with_scale else None
    _alg.check(_lib().pa_path_scores_f64(
        int(A.Type.DTW if dtw else A.Type.ALIGNMENT), int(A.Locality.__members__[locality.upper()]),
        int(A.Direction.__members__[direction.upper()]), B, paths.data_ptr(), poff.data_ptr(), plen.data_ptr(),
        base, soff.data_ptr(), S.stride(1), S.stride(2), None if g is None else g.ctypes.data, out.data_ptr(),
        None if scale is None else scale.data_ptr(), torch.cuda.current_stream().cuda_stream))
    return (scores, out, scale) if with_scale else (scores, out)


def _forward_paths(S, lengths, gap, locality, direction, dtw):
    """Scores and optimal paths of the pairs of S (device); returns (scores, paths, path
    lengths, device path offsets, layout flag)."""
    if not S.is_cuda or S.dtype != torch.float32 or S.dim() != 3:
        raise ValueError("S must be a (batch, len_s, len_t) float32 CUDA tensor")
    # any layout with unit stride along s or t is read in place; a transposed view
    # (stride 1 along s) is the fastest: each lane reads its 8 rows as one 32-byte sector
    if S.stride(1) != 1 and S.stride(2) != 1:
        S = S.contiguous()
    B, n_s, n_t = S.shape
    ss, st_ = S.stride(1), S.stride(2)
    solver, ln, scores, paths, plen, poff = _path_buffers(B, n_s, n_t, lengths, locality, direction, dtw, gap,
                                                          S.device, "the similarity tensor")
    offsets = S.storage_offset() + np.arange(B, dtype=np.int64) * S.stride(0)
    base = S.data_ptr() - S.storage_offset() * S.element_size()
    _alg.check(_lib().pa_solve_dense_paths(
        solver.handle, base, offsets.ctypes.data, ss, st_, B, n_s, n_t, ln.ctypes.data,
        scores.data_ptr(), paths.data_ptr(), poff.ctypes.data, plen.data_ptr()))
    return scores, paths, plen, _to_device(poff, S.device), ss == 1


def _path_buffers(B, n_s, n_t, lengths, locality, direction, dtw, gap, device, what):
    """The solver on the current stream, the (2, B) int32 lengths and the output buffers of a
    paths solve: scores, packed paths (2 (|s| + |t| + 2) entries per pair), path lengths and
    the host path offsets."""
    ln = np.ascontiguousarray(np.asarray(lengths).reshape(B, 2).T, dtype=np.int32)
    if (ln[0] > n_s).any() or (ln[1] > n_t).any() or (ln < 0).any():
        raise ValueError("lengths exceed " + what)
    solver = _solver(B, n_s, n_t, locality, direction, dtw, gap)
    stream = torch.cuda.current_stream()
    _alg.check(_lib().pa_solver_set_stream(solver.handle, ctypes.c_void_p(stream.cuda_stream)))
    sizes = 2 * (ln[0].astype(np.int64) + ln[1] + 2)
    poff = np.zeros(B, np.int64)
    poff[1:] = np.cumsum(sizes)[:-1]
    paths = torch.empty(int(sizes.sum()), dtype=torch.int32, device=device)
    plen = torch.zeros(B, dtype=torch.int32, device=device)
    scores = torch.empty(B, dtype=torch.float32, device=device)
    return solver, ln, scores, paths, plen, poff


def _series_paths(x, y, lengths, gap, locality, direction, dtw):
    """_forward_paths for S(u, v) = |x_u - y_v| of the series rows of x and y (contiguous
    float32 CUDA tensors): the kernel computes each cell, no matrix is formed."""
    B, n_s = x.shape
    n_t = y.shape[1]
    solver, ln, scores, paths, plen, poff = _path_buffers(B, n_s, n_t, lengths, locality, direction, dtw, gap,
                                                          x.device, "the series")
    _alg.check(_lib().pa_solve_series_paths(
        solver.handle, x.data_ptr(), x.stride(0), y.data_ptr(), y.stride(0), B, n_s, n_t, ln.ctypes.data,
        scores.data_ptr(), paths.data_ptr(), poff.ctypes.data, plen.data_ptr()))
    return scores, paths, plen, _to_device(poff, x.device)


def _gap_grads(dtw, linear, locality, direction, B, paths, plen, poff, grad):
    """d score / d (open, extend) summed over pairs (pa_path_gradients without dS)."""
    if dtw:
        return None, None
    A = _alg
    dgap = torch.empty((B, 4), dtype=torch.float32, device=grad.device)  # every pair writes its 4
    _alg.check(_lib().pa_path_gradients(
        int(A.Type.ALIGNMENT), int(A.Locality.__members__[locality.upper()]),
        int(A.Direction.__members__[direction.upper()]), B, paths.data_ptr(), poff.data_ptr(),
        plen.data_ptr(), grad.data_ptr(), None, None, 0, 0, dgap.data_ptr(),
        torch.cuda.current_stream().cuda_stream))
    # one reduction: (open_s + open_t, extend_s + extend_t) summed over pairs
    if linear:
        return dgap.sum(), None
    tot = dgap.view(B, 2, 2).sum(dim=(0, 1))
    return tot[0], tot[1]


class AlignmentScore(torch.autograd.Function):
    """Optimal alignment score of each pair; backward = path indicator and gap counts."""

    @staticmethod
    def forward(ctx, S, lengths, gap_open, gap_extend, locality, direction, dtw, linear):
        gap = None if dtw else ((float(gap_open), None) if linear else (float(gap_open), float(gap_extend)))
        scores, paths, plen, poff, transposed = _forward_paths(S, lengths, gap, locality, direction, dtw)
        ctx.save_for_backward(paths, plen, poff)
        ctx.meta = (S.shape, locality, direction, dtw, linear, transposed)
        return scores

    @staticmethod
    def backward(ctx, grad):
        paths, plen, poff = ctx.saved_tensors
        (B, n_s, n_t), locality, direction, dtw, linear, transposed = ctx.meta
        A = _alg
        grad = grad.contiguous().float()
        # dS in the layout S came in: a transposed view when S was one
        if transposed:
            dS = torch.zeros((B, n_t, n_s), dtype=torch.float32, device=grad.device).transpose(1, 2)
        else:
            dS = torch.zeros((B, n_s, n_t), dtype=torch.float32, device=grad.device)
        dgap = torch.zeros((B, 4), dtype=torch.float32, device=grad.device)
        offsets = torch.arange(B, dtype=torch.int64, device=grad.device) * (n_s * n_t)
        _alg.check(_lib().pa_path_gradients(
            int(A.Type.DTW if dtw else A.Type.ALIGNMENT), int(A.Locality.__members__[locality.upper()]),
            int(A.Direction.__members__[direction.upper()]), B, paths.data_ptr(), poff.data_ptr(),
            plen.data_ptr(), grad.data_ptr(), dS.data_ptr(), offsets.data_ptr(), dS.stride(1), dS.stride(2),
            dgap.data_ptr(), torch.cuda.current_stream().cuda_stream))
        tot = dgap.sum(dim=0)
        if dtw:
            d_open = d_ext = None
        elif linear:
            d_open, d_ext = tot[0] + tot[1] + tot[2] + tot[3], None
        else:
            d_open, d_ext = tot[0] + tot[2], tot[1] + tot[3]
        return dS, None, d_open, d_ext, None, None, None, None


def alignment_score(S, lengths, gap_open=None, gap_extend=None, locality="global", direction="maximize",
                    dtw=False):
    """Differentiable optimal scores of `batch` pairs.

    S: (batch, len_s, len_t) float32 CUDA tensor of similarities (distances when
    minimizing), padded; lengths: (batch, 2) of |s|, |t|.  Affine gaps w(k) = open +
    extend (k - 1) when both are given, linear w(k) = open * k when gap_extend is None;
    DTW ignores gaps.  gap_open/gap_extend may be tensors that require grad.
    """
    linear = gap_extend is None
    go = gap_open if isinstance(gap_open, torch.Tensor) else torch.tensor(float(gap_open or 0.0))
    ge = gap_extend if isinstance(gap_extend, torch.Tensor) else torch.tensor(float(gap_extend or 0.0))
    return AlignmentScore.apply(S, lengths, go, ge, locality, direction, dtw, linear)


SIM_TILE = 128  # rows of a tile of the tensor-core product (pa_simgemm.cu TM, TN)


def normalized_bf16(E, normalize=True, lengths=None, tiled=False):
    """The BF16 factor of E (batch, n, d) for the similarity product -- E / |E| per row when
    normalising -- and 1 / |E| per row, in one pass (pa_normalize_rows_bf16).  d is padded
    with zeros to a multiple of 16 (the tensor-core K step).  With ``lengths`` (batch,) the
    rows past each pair's length are zero and not read (pa_normalize_rows_bf16_lengths);
    with ``tiled`` only the rows the product's tiles read are written (up to each length
    rounded up to SIM_TILE; the rows beyond keep whatever the fresh tensor held), for a factor
    that only similarity_bf16 and the aligned rows of the backward read."""
    E = _pad16(E.contiguous().float())
    B, n, dim = E.shape
    Eb = torch.empty(E.shape, dtype=torch.bfloat16, device=E.device)
    inv = torch.empty(B * n, dtype=torch.float32, device=E.device)
    stream = torch.cuda.current_stream().cuda_stream
    if lengths is None:
        _alg.check(_lib().pa_normalize_rows_bf16(E.data_ptr(), B * n, dim, int(normalize), Eb.data_ptr(),
                                                 inv.data_ptr(), stream))
    else:
        ln = _to_device(np.minimum(np.asarray(lengths).reshape(B), n).astype(np.int32), E.device)
        if tiled:
            _alg.check(_lib().pa_normalize_rows_bf16_tiled(E.data_ptr(), B, n, dim, int(normalize), ln.data_ptr(),
                                                           SIM_TILE, Eb.data_ptr(), inv.data_ptr(), stream))
        else:
            _alg.check(_lib().pa_normalize_rows_bf16_lengths(E.data_ptr(), B, n, dim, int(normalize),
                                                             ln.data_ptr(), Eb.data_ptr(), inv.data_ptr(), stream))
    return Eb, inv


class CosineSimilarity(torch.autograd.Function):
    """S = <en_s, en_t> with en = E / |E|, the product on the tensor cores.  Backward: the
    dense route, dEn_s = dS en_t and dEn_t = dS^T en_s (the BF16 cast passes gradients
    through), then the normalisation backward (g - (g . en) en) / |E|."""

    @staticmethod
    def forward(ctx, Es, Et, lengths):
        B, n_s, d = Es.shape
        n_t = Et.shape[1]
        ln = None if lengths is None else np.asarray(lengths).reshape(B, 2)
        Esb, inv_s = normalized_bf16(Es, True, None if ln is None else ln[:, 0])  # padding rows: zero
        Etb, inv_t = normalized_bf16(Et, True, None if ln is None else ln[:, 1])
        if lengths is None:
            lengths = np.tile(np.array([[n_s, n_t]], np.int32), (B, 1))
            out = None
        else:
            out = torch.zeros((B, n_t, n_s), dtype=torch.float32, device=Es.device)
        ctx.save_for_backward(Esb, Etb, inv_s, inv_t)
        ctx.d = d
        return similarity_bf16(Esb, Etb, lengths, out=out)

    @staticmethod
    def backward(ctx, dS):
        Esb, Etb, inv_s, inv_t = ctx.saved_tensors
        B, n_s, dp = Esb.shape
        n_t = Etb.shape[1]
        en_s, en_t = Esb.float(), Etb.float()
        g_s = torch.bmm(dS.float(), en_t)
        g_t = torch.bmm(dS.float().transpose(1, 2), en_s)
        inv_s = inv_s.view(B, n_s, 1)
        inv_t = inv_t.view(B, n_t, 1)
        # en here is the BF16 factor; the normalisation backward uses the exact en = E / |E|
        # only through (g . en) en, where the BF16 rounding is below float32 noise of g
        d_s = (g_s - (g_s * en_s).sum(-1, keepdim=True) * en_s) * inv_s
        d_t = (g_t - (g_t * en_t).sum(-1, keepdim=True) * en_t) * inv_t
        return d_s[..., :ctx.d], d_t[..., :ctx.d], None


def cosine_similarity_batch(Es, Et, lengths=None):
    """S = cos(E_s, E_t) per pair: L2-normalised embeddings multiplied in BF16 with FP32
    accumulation on the tensor cores.  Es: (batch, len_s, d), Et: (batch, len_t, d);
    lengths (batch, 2) limits the product to each pair's cells (the rest of S is zero).
    Returned as a transposed view of S^T (stride 1 along s), the layout the DP reads
    fastest.  Differentiable with respect to Es and Et."""
    return CosineSimilarity.apply(Es, Et, lengths)


class EmbeddingAlignmentScore(torch.autograd.Function):
    """Alignment score of S = <en_s, en_t^T> for per-token embeddings (en = E/|E| for the
    cosine, E for the dot product), the product in BF16 with FP32 accumulation.  The
    backward walks the optimal paths and writes the gradients of the aligned rows of E
    directly, through the normalisation (pa_path_embedding_gradients): O(path * d) work
    instead of a dense dS, two batched products and a dense normalisation backward."""

    @staticmethod
    def forward(ctx, Es, Et, lengths, gap_open, gap_extend, locality, direction, linear, normalize):
        dim_in = Es.shape[-1]
        Es = _pad16(Es.contiguous().float())
        Et = _pad16(Et.contiguous().float())
        ln = np.asarray(lengths).reshape(Es.shape[0], 2)
        # rows past a pair's length: zero up to the product's tile, not read, not written beyond
        Esb, inv_s = normalized_bf16(Es, normalize, ln[:, 0], tiled=True)
        Etb, inv_t = normalized_bf16(Et, normalize, ln[:, 1], tiled=True)
        # S^T = en_t en_s^T on the tensor cores, only the cells inside the lengths; its
        # transposed view is S with stride 1 along s
        S = similarity_bf16(Esb, Etb, lengths)
        gap = (float(gap_open), None) if linear else (float(gap_open), float(gap_extend))
        scores, paths, plen, poff, _ = _forward_paths(S, lengths, gap, locality, direction, False)
        ctx.save_for_backward(Es, Et, Esb, Etb, inv_s, inv_t, paths, plen, poff)
        ctx.meta = (locality, direction, linear, normalize)
        ctx.dim_in = dim_in
        return scores

    @staticmethod
    def backward(ctx, grad):
        Es, Et, Esb, Etb, inv_s, inv_t, paths, plen, poff = ctx.saved_tensors
        locality, direction, linear, normalize = ctx.meta
        grad = grad.contiguous().float()
        B, n_s, dim = Es.shape
        n_t = Et.shape[1]
        d_in = ctx.dim_in
        dEs = torch.empty_like(Es)  # every row is written: the aligned ones, zeros elsewhere
        dEt = torch.empty_like(Et)
        _alg.check(_lib().pa_path_embedding_gradients_full(
            B, dim, int(normalize), paths.data_ptr(), poff.data_ptr(), plen.data_ptr(), grad.data_ptr(),
            Es.data_ptr(), Et.data_ptr(), Esb.data_ptr(), Etb.data_ptr(), inv_s.data_ptr(), inv_t.data_ptr(),
            n_s, n_t, dEs.data_ptr(), dEt.data_ptr(), torch.cuda.current_stream().cuda_stream))
        d_open, d_ext = _gap_grads(False, linear, locality, direction, B, paths, plen, poff, grad)
        return dEs[..., :d_in], dEt[..., :d_in], None, d_open, d_ext, None, None, None, None


def embedding_alignment_score(Es, Et, lengths, gap_open, gap_extend=None, locality="global",
                              direction="maximize", normalize=True):
    """Differentiable alignment scores on the cosine (normalize=True) or dot similarity of
    per-token embeddings Es (batch, len_s, d) and Et (batch, len_t, d), padded."""
    linear = gap_extend is None
    go = gap_open if isinstance(gap_open, torch.Tensor) else torch.tensor(float(gap_open))
    ge = gap_extend if isinstance(gap_extend, torch.Tensor) else torch.tensor(float(gap_extend or 0.0))
    return EmbeddingAlignmentScore.apply(Es, Et, lengths, go, ge, locality, direction, linear, normalize)


class SeriesDTW(torch.autograd.Function):
    """DTW score (minimize) of series pairs with d(u, v) = |x_u - y_v|; the backward walks
    the optimal paths (pa_path_series_gradients)."""

    @staticmethod
    def forward(ctx, x, y, lengths):
        x = x.contiguous().float()
        y = y.contiguous().float()
        if x.dim() != 2 or y.dim() != 2 or x.shape[0] != y.shape[0] or not x.is_cuda or y.device != x.device:
            raise ValueError("x, y must be (batch, len) CUDA tensors on one device")
        scores, paths, plen, poff = _series_paths(x, y, lengths, None, "global", "minimize", True)
        ctx.save_for_backward(x, y, paths, plen, poff)
        return scores

    @staticmethod
    def backward(ctx, grad):
        x, y, paths, plen, poff = ctx.saved_tensors
        grad = grad.contiguous().float()
        dx = torch.zeros_like(x)
        dy = torch.zeros_like(y)
        _alg.check(_lib().pa_path_series_gradients(
            x.shape[0], paths.data_ptr(), poff.data_ptr(), plen.data_ptr(), grad.data_ptr(), x.data_ptr(),
            y.data_ptr(), x.shape[1], y.shape[1], dx.data_ptr(), dy.data_ptr(),
            torch.cuda.current_stream().cuda_stream))
        return dx, dy, None


def dtw_series_score(x, y, lengths):
    """Differentiable DTW (minimize, |x_u - y_v|) of series x (batch, len_s), y (batch, len_t)."""
    return SeriesDTW.apply(x, y, lengths)
