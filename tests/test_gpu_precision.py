"""Score error of the similarity-matrix path against the FP64 oracle (needs a GPU).

Embedding alignment: 48 pairs with lengths uniform in [32, 512], per-token embeddings
d = 256 drawn N(0, 1) and L2-normalised, S = cosine on the tensor cores (BF16 factors, FP32
accumulation), global affine gaps open 0.5 / extend 0.1 maximised with the float32 DP, and
DTW (minimise) on 1 - cos (written by the same kernel's epilogue).  Three errors:

* DP: the float32 DP on our S against the FP64 oracle DP on the same S (as float64)
  -- the accumulation error of the DP alone; bound 1e-5.
* product + DP: against the FP64 oracle on the FP64 product of the same BF16 factors -- adds
  the FP32 accumulation of the tensor-core product.  Global scores of random embeddings
  can sit near zero (gap costs cancel the aligned similarities), where an error relative
  to |score| says nothing about the arithmetic; this one is bounded (1e-5) relative to the
  magnitude of the terms the score sums, sum |S| over the aligned cells plus the gap
  costs, and its |score|-relative value is printed beside it.
* replay: the FP64 re-evaluation of our recovered path on the GPU (pa_path_scores_f64)
  against our float32 score; bound 1e-5, and it equals the oracle's FP64 score wherever the
  two optimal paths coincide.

The error of BF16-quantising the embeddings themselves (FP64 product of the unrounded
normalised embeddings) is printed for the record, not bounded: it is the precision choice
of the form, not an arithmetic error of the kernels.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPEN, EXT = 0.5, 0.1


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from pyalign_gb300 import build
    build.build()
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device visible")
    from pyalign_gb300 import autograd
    import oracle.algorithm as oalg
    L = ctypes.CDLL(oalg.build())
    vp, i32 = ctypes.c_void_p, ctypes.c_int32
    L.pao_solve_f64.restype = i32
    L.pao_solve_f64.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp, vp, vp]
    return torch, autograd, oalg, L


def _f64(oalg, L, S, dtw):
    ls, lt = S.shape
    o = oalg._Options()
    o.type = 1 if dtw else 0
    o.direction = 0 if dtw else 1
    o.detail, o.count = 1, 0
    o.locality = 1
    o.remove_dup = 1
    o.cap_s, o.cap_t = ls, lt
    gaps = np.zeros(6, np.float64)
    if not dtw:
        o.gap_kind = 1
        gaps[2] = gaps[4] = EXT
        gaps[3] = gaps[5] = OPEN - EXT
    S = np.ascontiguousarray(S, dtype=np.float64)
    sc = ctypes.c_double(0)
    path = np.zeros((ls + lt + 4, 2), np.int32)
    n = ctypes.c_int32(0)
    assert L.pao_solve_f64(ctypes.addressof(o), gaps.ctypes.data, None, None, ls, lt, S.ctypes.data,
                           ctypes.addressof(sc), path.ctypes.data, ctypes.addressof(n))
    return sc.value, path[:n.value]


def _scale(S, path, score, dtw):
    """sum |S| over the cells the score adds (aligned cells; every visited cell for DTW)
    plus the total gap cost of the path."""
    tot = mag = 0.0
    for q in range(len(path) - 1):
        u0, v0 = path[q]
        u1, v1 = path[q + 1]
        if u0 < 0 or v0 < 0:
            break
        if dtw or (u1 == u0 - 1 and v1 == v0 - 1):
            tot += S[u0, v0]
            mag += abs(S[u0, v0])
    return mag + abs(tot - score)


def test_embedding_alignment_error_vs_fp64_oracle(env):
    torch, ag, oalg, L = env
    rng = np.random.default_rng(1004)
    B, n, d = 48, 512, 256
    lengths = rng.integers(32, 513, size=(B, 2))
    g = torch.Generator(device="cuda").manual_seed(1004)
    Es = torch.randn(B, n, d, device="cuda", generator=g)
    Et = torch.randn(B, n, d, device="cuda", generator=g)
    S = ag.cosine_similarity_batch(Es, Et, lengths)          # (B, n, n) view, zero padding
    assert ag.tensor_core_status() == 0
    Sh = S.double().cpu().numpy()
    Esb, _ = ag.normalized_bf16(Es)      # the BF16 factors the kernel multiplied
    Etb, _ = ag.normalized_bf16(Et)
    Sq = torch.bmm(Esb.double(), Etb.double().transpose(1, 2)).cpu().numpy()
    en_s = torch.nn.functional.normalize(Es.double(), dim=-1)
    en_t = torch.nn.functional.normalize(Et.double(), dim=-1)
    Sx = torch.bmm(en_s, en_t.transpose(1, 2)).cpu().numpy()

    report = {}
    for dtw in (False, True):
        if dtw:
            D = ag.similarity_bf16(Esb, Etb, lengths, out=torch.ones((B, n, n), device="cuda"),
                                   alpha=-1.0, beta=1.0)
            sc32, rep64 = ag.path_scores_f64(D, lengths, locality="global", direction="minimize", dtw=True)
            Mh = D.double().cpu().numpy()    # the float32 distances the DP read
        else:
            Mh = Sh
            sc32, rep64 = ag.path_scores_f64(S, lengths, OPEN, EXT, "global", "maximize")
        sc32 = sc32.double().cpu().numpy()
        rep64 = rep64.cpu().numpy()
        e_dp, e_gemm, e_gemm_s, e_rep, e_bf16, e_bf16_s, same = [], [], [], [], [], [], 0
        for k, (ls, lt) in enumerate(lengths):
            f = (lambda M: 1.0 - M) if dtw else (lambda M: M)
            o_same, _ = _f64(oalg, L, Mh[k, :ls, :lt], dtw)
            o_q, path_q = _f64(oalg, L, f(Sq[k, :ls, :lt]), dtw)
            o_x, path_x = _f64(oalg, L, f(Sx[k, :ls, :lt]), dtw)
            e_dp.append(abs(sc32[k] - o_same) / abs(o_same))
            e_gemm.append(abs(sc32[k] - o_q) / _scale(f(Sq[k, :ls, :lt]), path_q, o_q, dtw))
            e_gemm_s.append(abs(sc32[k] - o_q) / abs(o_q))
            e_rep.append(abs(sc32[k] - rep64[k]) / abs(rep64[k]))
            e_bf16.append(abs(sc32[k] - o_x) / _scale(f(Sx[k, :ls, :lt]), path_x, o_x, dtw))
            e_bf16_s.append(abs(sc32[k] - o_x) / abs(o_x))
            if abs(rep64[k] - o_same) <= 1e-12 * abs(o_same):
                same += 1
        name = "dtw" if dtw else "gotoh"
        report[name] = {"dp": max(e_dp), "replay": max(e_rep), "product+dp (term scale)": max(e_gemm),
                        "product+dp (|score|)": max(e_gemm_s), "bf16 inputs (term scale)": max(e_bf16),
                        "bf16 inputs (|score|)": max(e_bf16_s), "min |score|": float(np.abs(sc32).min()),
                        "paths equal to the fp64 optimum": same}
        print(name, report[name])
        assert max(e_dp) <= 1e-5, (name, max(e_dp))
        assert max(e_rep) <= 1e-5, (name, max(e_rep))
        assert max(e_gemm) <= 1e-5, (name, max(e_gemm))
        assert same >= B - 2, (name, same)   # optimal paths coincide but for near-ties
    print("relative score error (max over pairs):", report)


def test_precision_report_at_size(env):
    """1,024 pairs of the precision workload (L ~ U[32, 512], d = 256, cos on the tensor
    cores, global Gotoh 0.5/0.1 and DTW on 1 - cos): the float32 DP against the FP64 oracle
    DP on the same S, for every pair.  Bound: the error relative to the magnitude of the
    terms the score sums is <= 1e-5 for every pair.  Relative to |score| the pairs above 1e-5
    are reported with their |score| and summed-terms magnitude: global scores of random
    embeddings can nearly cancel, and there the float32 rounding of the terms, not of the
    score, sets the error.  DTW scores are sums of positive distances: bounded by 1e-5 of
    |score| for every pair."""
    torch, ag, oalg, _ = env
    rng = np.random.default_rng(1044)
    B, n, d = 1024, 512, 256
    lengths = rng.integers(32, n + 1, size=(B, 2))
    g = torch.Generator(device="cuda").manual_seed(1044)
    Es = torch.randn(B, n, d, device="cuda", generator=g)
    Et = torch.randn(B, n, d, device="cuda", generator=g)
    S = ag.cosine_similarity_batch(Es, Et, lengths)
    assert ag.tensor_core_status() == 0
    sc32, rep64 = ag.path_scores_f64(S, lengths, OPEN, EXT, "global", "maximize")
    Sh = S.cpu().numpy()
    o64, scale = oalg.batch_f64(Sh, lengths[:, 0], lengths[:, 1], open_=OPEN, extend=EXT)
    sc = sc32.double().cpu().numpy()
    err = np.abs(sc - o64)
    rel_s = err / np.abs(o64)
    rel_t = err / scale
    over = rel_s > 1e-5
    print(f"gotoh: max rel |score| {rel_s.max():.3e}, over 1e-5: {int(over.sum())}/{B}, "
          f"max rel terms {rel_t.max():.3e}")
    assert rel_t.max() <= 1e-5, rel_t.max()
    print("  (|score|, summed terms) of those:", list(zip(np.abs(o64[over]).round(4), scale[over].round(2))))
    rep = np.abs(sc - rep64.cpu().numpy()) / scale
    assert rep.max() <= 1e-5, rep.max()

    Esb, _ = ag.normalized_bf16(Es)
    Etb, _ = ag.normalized_bf16(Et)
    D = ag.similarity_bf16(Esb, Etb, lengths, out=torch.ones((B, n, n), device="cuda"), alpha=-1.0, beta=1.0)
    dsc, _ = ag.path_scores_f64(D, lengths, locality="global", direction="minimize", dtw=True)
    d64, _ = oalg.batch_f64(D.cpu().numpy(), lengths[:, 0], lengths[:, 1], dtw=True, direction="minimize")
    drel = np.abs(dsc.double().cpu().numpy() - d64) / np.abs(d64)
    print(f"dtw: max rel |score| {drel.max():.3e}")
    assert drel.max() <= 1e-5, drel.max()

