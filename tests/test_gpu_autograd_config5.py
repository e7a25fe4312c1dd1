"""Gradient checks of the differentiation form at its stated size (needs a GPU).

Workload: 4,096 pairs with |s|, |t| ~ U[64, 256], per-token embeddings d = 128 drawn
N(0, 1), S = cosine on the tensor cores (BF16 factors, FP32 accumulation), global affine
gaps open 0.5 / extend 0.1, maximised.  One forward + backward over the whole batch; then,
on pairs sampled from it:

1. dScore/dS and dScore/d(open, extend) against central finite differences (eps = 1e-3) of
   the oracle's FP64 twin on the same S, on 64 tie-free pairs: a pair counts as tie-free
   when the FP64 optimal path is the same at every perturbed input, so the score is
   differentiable there and the finite difference is its derivative.  Bound 1e-6 (dS) and
   1e-5 (the gap sums).
2. dScore/dE_s and dScore/dE_t against central finite differences of the FP64 objective --
   cosine normalisation and product in FP64, the FP64 DP -- on a handful of coordinates of
   aligned and unaligned rows.  The backward differentiates through the BF16 factors the
   product used, so the bound is BF16-level: 2% of the derivative plus 5e-5.
"""

import concurrent.futures
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPEN, EXT = 0.5, 0.1
EPS = 1e-3


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


def _f64(oalg, L, S, gap=(OPEN, EXT)):
    """FP64 score and optimal path of one pair, global affine (maximize)."""
    ls, lt = S.shape
    o = oalg._Options()
    o.type, o.direction, o.detail, o.count, o.locality, o.remove_dup, o.gap_kind = 0, 1, 1, 0, 1, 1, 1
    o.cap_s, o.cap_t = ls, lt
    gaps = np.zeros(6, np.float64)
    gaps[2] = gaps[4] = gap[1]
    gaps[3] = gaps[5] = gap[0] - gap[1]
    S = np.ascontiguousarray(S, dtype=np.float64)
    sc = ctypes.c_double(0)
    path = np.zeros((ls + lt + 4, 2), np.int32)
    n = ctypes.c_int32(0)
    assert L.pao_solve_f64(ctypes.addressof(o), gaps.ctypes.data, None, None, ls, lt, S.ctypes.data,
                           ctypes.addressof(sc), path.ctypes.data, ctypes.addressof(n))
    return sc.value, path[:n.value].copy()


def _aligned(path):
    return [(int(u0), int(v0)) for (u0, v0), (u1, v1) in zip(path[:-1], path[1:])
            if u0 >= 0 and v0 >= 0 and u1 == u0 - 1 and v1 == v0 - 1]


def _workload(torch, ag, B=4096, d=128, seed=1005):
    rng = np.random.default_rng(seed)
    lengths = rng.integers(64, 257, size=(B, 2))
    g = torch.Generator(device="cuda").manual_seed(seed)
    Es = torch.randn(B, 256, d, device="cuda", generator=g)
    Et = torch.randn(B, 256, d, device="cuda", generator=g)
    return rng, lengths, Es, Et


def test_central_fd_on_64_tie_free_pairs(env):
    torch, ag, oalg, L = env
    rng, lengths, Es, Et = _workload(torch, ag)
    B = len(lengths)
    S = ag.cosine_similarity_batch(Es, Et, lengths).contiguous().requires_grad_(True)
    go = torch.tensor(OPEN, requires_grad=True)
    ge = torch.tensor(EXT, requires_grad=True)
    scores = ag.alignment_score(S, lengths, go, ge, "global", "maximize")
    w = torch.from_numpy(rng.normal(size=B).astype(np.float32)).cuda()   # a weighted sum: per-pair grads
    (scores * w).sum().backward()
    dS = S.grad.cpu().numpy()
    Sh = S.detach().cpu().numpy()
    wh = w.cpu().numpy().astype(np.float64)

    def check(k):
        ls, lt = lengths[k]
        base = Sh[k, :ls, :lt].astype(np.float64)
        sc, path = _f64(oalg, L, base)
        al = _aligned(path)
        cells = al[:: max(1, len(al) // 6)][:6] + [(int(rng_k.integers(0, ls)), int(rng_k.integers(0, lt)))
                                                   for rng_k in [np.random.default_rng(k)] for _ in range(6)]
        out = []
        for (i, j) in cells:
            hi, lo = base.copy(), base.copy()
            hi[i, j] += EPS
            lo[i, j] -= EPS
            (s_hi, p_hi), (s_lo, p_lo) = _f64(oalg, L, hi), _f64(oalg, L, lo)
            if not (np.array_equal(p_hi, path) and np.array_equal(p_lo, path)):
                return None                                   # a tie within eps: not tie-free
            out.append((i, j, (s_hi - s_lo) / (2 * EPS)))
        gaps = []
        for gp, gm in (((OPEN + EPS, EXT), (OPEN - EPS, EXT)), ((OPEN, EXT + EPS), (OPEN, EXT - EPS))):
            (s_hi, p_hi), (s_lo, p_lo) = _f64(oalg, L, base, gp), _f64(oalg, L, base, gm)
            if not (np.array_equal(p_hi, path) and np.array_equal(p_lo, path)):
                return None
            gaps.append((s_hi - s_lo) / (2 * EPS))
        return k, out, gaps

    sample = np.random.default_rng(77).permutation(B)[:160]
    with concurrent.futures.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        results = [r for r in ex.map(check, sample) if r is not None][:64]
    assert len(results) == 64, f"only {len(results)} tie-free pairs among 160 sampled"
    for k, cells, _ in results:
        for i, j, fd in cells:
            assert abs(fd * wh[k] - dS[k, i, j]) < 1e-6, (k, i, j, fd * wh[k], dS[k, i, j])
    # the gap gradients are sums over all pairs; check the sampled pairs' share against a
    # backward of the same pairs alone
    idx = np.array([r[0] for r in results])
    S2 = S.detach()[torch.from_numpy(idx).cuda()].contiguous().requires_grad_(True)
    go2 = torch.tensor(OPEN, requires_grad=True)
    ge2 = torch.tensor(EXT, requires_grad=True)
    (ag.alignment_score(S2, lengths[idx], go2, ge2, "global", "maximize") * w[torch.from_numpy(idx).cuda()]).sum().backward()
    d_open = sum(r[2][0] * wh[r[0]] for r in results)
    d_ext = sum(r[2][1] * wh[r[0]] for r in results)
    assert abs(go2.grad.item() - d_open) < 1e-5 * max(1.0, abs(d_open)), (go2.grad.item(), d_open)
    assert abs(ge2.grad.item() - d_ext) < 1e-5 * max(1.0, abs(d_ext)), (ge2.grad.item(), d_ext)


def test_embedding_gradients_central_fd(env):
    torch, ag, oalg, L = env
    rng, lengths, Es, Et = _workload(torch, ag)
    a = Es.clone().requires_grad_(True)
    b = Et.clone().requires_grad_(True)
    ag.embedding_alignment_score(a, b, lengths, OPEN, EXT, "global", "maximize").sum().backward()
    ga, gb = a.grad.cpu().numpy(), b.grad.cpu().numpy()
    Eh, Fh = Es.cpu().numpy().astype(np.float64), Et.cpu().numpy().astype(np.float64)

    def cos(E, F):
        return (E / np.linalg.norm(E, axis=1, keepdims=True)) @ (F / np.linalg.norm(F, axis=1, keepdims=True)).T

    checked, pairs_done = 0, 0
    for k in np.random.default_rng(5).permutation(len(lengths))[:12]:
        ls, lt = lengths[k]
        E, F = Eh[k, :ls], Fh[k, :lt]
        sc, path = _f64(oalg, L, cos(E, F))
        al = _aligned(path)
        rows_s = [al[len(al) // 3][0], al[2 * len(al) // 3][0]]
        rows_t = [al[len(al) // 2][1]]
        free_s = sorted(set(range(ls)) - {u for u, _ in al})
        rows_s += free_s[:1]                                  # an unaligned row: gradient 0
        coords, stable = [], True
        for side, rows in (("s", rows_s), ("t", rows_t)):
            for i in rows:
                for c in np.random.default_rng(int(k) * 7 + i).choice(128, 3, replace=False):
                    vals = []
                    for sgn in (1, -1):
                        E2, F2 = E.copy(), F.copy()
                        (E2 if side == "s" else F2)[i, c] += sgn * EPS
                        s2, p2 = _f64(oalg, L, cos(E2, F2))
                        vals.append(s2)
                        stable &= bool(np.array_equal(p2, path))
                    coords.append((side, i, c, (vals[0] - vals[1]) / (2 * EPS)))
        if not stable:
            continue                                          # a tie within eps: not differentiable here
        for side, i, c, fd in coords:
            g = (ga if side == "s" else gb)[k, i, c]
            assert abs(g - fd) <= 2e-2 * abs(fd) + 5e-5, (side, k, i, c, g, fd)
            checked += 1
        pairs_done += 1
        if pairs_done == 4:
            break
    assert pairs_done == 4 and checked >= 40, (pairs_done, checked)
