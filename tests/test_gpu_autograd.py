"""Gradients of the optimal alignment score (the differentiation form; needs a GPU).

1. dScore/dS from pa_path_gradients equals the indicator of the aligned cells of the
   float32 oracle's optimal path (every visited cell for DTW) -- exactly, and the scores
   are bit-identical.
2. Central finite differences in FP64 (eps = 1e-3, the oracle's FP64 twin) on tie-free
   continuous inputs agree with dScore/dS and dScore/d(open, extend) to 1e-6.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_ag():
    torch = pytest.importorskip("torch")
    from pyalign_gb300 import build
    build.build()
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device visible")
    from pyalign_gb300 import autograd
    return torch, autograd


@pytest.fixture(scope="module")
def f64():
    import oracle.algorithm as oalg
    L = ctypes.CDLL(oalg.build())
    vp, i32 = ctypes.c_void_p, ctypes.c_int32
    L.pao_solve_f64.restype = i32
    L.pao_solve_f64.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp, vp, vp]
    return oalg, L


def _oracle_f64(f64, S, ls, lt, locality, direction, dtw, gap):
    """FP64 score and path of one pair (S: ls x lt float64)."""
    oalg, L = f64
    o = oalg._Options()
    o.type = 1 if dtw else 0
    o.direction = 1 if direction == "maximize" else 0
    o.detail, o.count = 1, 0
    o.locality = {"local": 0, "global": 1, "semiglobal": 2}[locality]
    o.remove_dup = 1
    o.cap_s, o.cap_t = ls, lt
    gaps = np.zeros(6, np.float64)
    if not dtw:
        if gap[1] is None:
            o.gap_kind = 0
            gaps[0] = gaps[1] = gap[0]
        else:
            o.gap_kind = 1
            op, ex = gap
            gaps[2] = gaps[4] = ex            # Gotoh u = extend
            gaps[3] = gaps[5] = op - ex       # Gotoh v = open - extend
    S = np.ascontiguousarray(S, dtype=np.float64)
    sc = ctypes.c_double(0)
    path = np.zeros((ls + lt + 4, 2), np.int32)
    n = ctypes.c_int32(0)
    ok = L.pao_solve_f64(ctypes.addressof(o), gaps.ctypes.data, None, None, ls, lt, S.ctypes.data,
                         ctypes.addressof(sc), path.ctypes.data, ctypes.addressof(n))
    assert ok
    return sc.value, path[:n.value]


def _oracle_f32(S, ls, lt, locality, direction, dtw, gap, cap):
    """Float32 score and path of one pair from the oracle (the reference's arithmetic).

    `cap` is the solver capacity: for non-integer gap costs the affine border vector
    depends on it through its linspace (solver.h:2876-2880), so it must match the GPU
    solver's (the padded shape of S)."""
    import types
    import oracle.algorithm as oalg
    gc = None
    if not dtw:
        from _cases import Gap
        gc = Gap("linear", gap[0]) if gap[1] is None else Gap("affine", gap[0], gap[1])
    d = {"solver": oalg.Type.DTW if dtw else oalg.Type.ALIGNMENT,
         "direction": oalg.Direction.__members__[direction.upper()], "batch": False, "return_dup": False,
         "locality": oalg.Locality.__members__[locality.upper()],
         "codomain": types.SimpleNamespace(detail=oalg.Detail.SOLUTION, count=oalg.Count.ONE),
         "gap_cost": gc}
    solver = oalg.m16.create_solver(cap[0], cap[1], oalg.m16.create_options(d))
    sol = solver.solve_for_solution(np.ascontiguousarray(S, dtype=np.float32)[:, :, None],
                                    np.array([[ls], [lt]], np.uint16))[0]
    return sol.score, np.asarray(sol.path, dtype=np.int64)


def _indicator(path, ls, lt, dtw):
    ind = np.zeros((ls, lt), np.float64)
    for q in range(len(path) - 1):
        u0, v0 = path[q]
        u1, v1 = path[q + 1]
        if u0 < 0 or v0 < 0:
            break
        if dtw or (u1 == u0 - 1 and v1 == v0 - 1):
            ind[u0, v0] += 1
    return ind


CASES = [("global", "maximize", False, (0.5, 0.1)), ("local", "maximize", False, (1.0, 0.25)),
         ("semiglobal", "maximize", False, (0.75, 0.2)), ("global", "minimize", False, (0.5, 0.1)),
         ("global", "maximize", False, (0.4, None)), ("global", "minimize", True, None)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-{'dtw' if c[2] else 'gap'}")
def test_path_indicator_matches_oracle_path(torch_ag, f64, case):
    torch, ag = torch_ag
    locality, direction, dtw, gap = case
    rng = np.random.default_rng(17)
    B, n = 24, 48
    lengths = np.stack([rng.integers(1, n + 1, B), rng.integers(1, n + 1, B)], axis=1)
    if dtw:
        x = np.cumsum(rng.normal(size=(B, n)), axis=1)
        y = np.cumsum(rng.normal(size=(B, n)), axis=1)
        S = np.abs(x[:, :, None] - y[:, None, :]).astype(np.float32)
    else:
        S = rng.normal(size=(B, n, n)).astype(np.float32)
    St = torch.from_numpy(S).cuda().requires_grad_(True)
    go = torch.tensor(gap[0] if gap else 0.0, requires_grad=not dtw)
    ge = torch.tensor(gap[1], requires_grad=True) if gap and gap[1] is not None else None
    scores = ag.alignment_score(St, lengths, go, ge, locality, direction, dtw)
    scores.sum().backward()
    dS = St.grad.cpu().numpy()
    for k in range(B):
        ls, lt = lengths[k]
        sc, path = _oracle_f32(S[k, :ls, :lt], ls, lt, locality, direction, dtw, gap, (n, n))
        ind = _indicator(path, ls, lt, dtw)
        assert np.array_equal(dS[k, :ls, :lt], ind), k
        assert not dS[k, ls:, :].any() and not dS[k, :, lt:].any()
        assert scores[k].item() == sc, (k, scores[k].item(), sc)
        sc64, _ = _oracle_f64(f64, S[k, :ls, :lt], ls, lt, locality, direction, dtw, gap)
        assert abs(sc - sc64) <= 1e-5 * max(1.0, abs(sc64)), (sc, sc64)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}-{'dtw' if c[2] else 'gap'}")
def test_central_finite_differences_fp64(torch_ag, f64, case):
    torch, ag = torch_ag
    locality, direction, dtw, gap = case
    rng = np.random.default_rng(91)
    B, n, eps = 8, 24, 1e-3
    lengths = np.stack([rng.integers(8, n + 1, B), rng.integers(8, n + 1, B)], axis=1)
    S = rng.normal(size=(B, n, n)).astype(np.float32)
    if dtw:
        S = np.abs(S)
    St = torch.from_numpy(S).cuda().requires_grad_(True)
    go = torch.tensor(gap[0] if gap else 0.0, requires_grad=not dtw)
    ge = torch.tensor(gap[1], requires_grad=True) if gap and gap[1] is not None else None
    ag.alignment_score(St, lengths, go, ge, locality, direction, dtw).sum().backward()
    dS = St.grad.cpu().numpy()
    d_open_fd = d_ext_fd = 0.0
    for k in range(B):
        ls, lt = lengths[k]
        base = S[k, :ls, :lt].astype(np.float64)
        cells = [(int(rng.integers(0, ls)), int(rng.integers(0, lt))) for _ in range(12)]
        _, path = _oracle_f64(f64, base, ls, lt, locality, direction, dtw, gap)
        cells += [tuple(p) for p in path if p[0] >= 0 and p[1] >= 0][:12]
        for (i, j) in cells:
            hi, lo = base.copy(), base.copy()
            hi[i, j] += eps
            lo[i, j] -= eps
            fd = (_oracle_f64(f64, hi, ls, lt, locality, direction, dtw, gap)[0] -
                  _oracle_f64(f64, lo, ls, lt, locality, direction, dtw, gap)[0]) / (2 * eps)
            assert abs(fd - dS[k, i, j]) < 1e-6, (k, i, j, fd, dS[k, i, j])
        if not dtw:
            g2 = (gap[0] + eps, gap[1]) if gap[1] is not None else (gap[0] + eps, None)
            g1 = (gap[0] - eps, gap[1]) if gap[1] is not None else (gap[0] - eps, None)
            d_open_fd += (_oracle_f64(f64, base, ls, lt, locality, direction, dtw, g2)[0] -
                          _oracle_f64(f64, base, ls, lt, locality, direction, dtw, g1)[0]) / (2 * eps)
            if gap[1] is not None:
                e2 = (gap[0], gap[1] + eps)
                e1 = (gap[0], gap[1] - eps)
                d_ext_fd += (_oracle_f64(f64, base, ls, lt, locality, direction, dtw, e2)[0] -
                             _oracle_f64(f64, base, ls, lt, locality, direction, dtw, e1)[0]) / (2 * eps)
    if not dtw:
        assert abs(go.grad.item() - d_open_fd) < 1e-5, (go.grad.item(), d_open_fd)
        if ge is not None:
            assert abs(ge.grad.item() - d_ext_fd) < 1e-5, (ge.grad.item(), d_ext_fd)


def test_embedding_gradients_flow(torch_ag):
    """S = cos(E_s, E_t) in BF16 with FP32 accumulation; gradients reach the embeddings."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(5)
    Es = torch.randn(16, 40, 64, device="cuda", generator=g, requires_grad=True)
    Et = torch.randn(16, 36, 64, device="cuda", generator=g, requires_grad=True)
    lengths = np.full((16, 2), (40, 36))
    S = ag.cosine_similarity_batch(Es, Et)
    ag.alignment_score(S, lengths, 0.5, 0.1).sum().backward()
    assert torch.isfinite(Es.grad).all() and Es.grad.abs().sum() > 0
    assert torch.isfinite(Et.grad).all() and Et.grad.abs().sum() > 0


def test_fused_embedding_gradients_match_dense_route(torch_ag):
    """embedding_alignment_score's path-walk backward (dot similarity) equals dS @ Et with dS
    the path indicator of the dense route (one aligned j per i, so the sums are single
    terms)."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(9)
    B, ns, nt, d = 32, 50, 44, 64
    Es = torch.randn(B, ns, d, device="cuda", generator=g)
    Et = torch.randn(B, nt, d, device="cuda", generator=g)
    rng = np.random.default_rng(4)
    lengths = np.stack([rng.integers(1, ns + 1, B), rng.integers(1, nt + 1, B)], axis=1)
    for locality in ("global", "local", "semiglobal"):
        a = Es.clone().requires_grad_(True)
        b = Et.clone().requires_grad_(True)
        go = torch.tensor(0.5, requires_grad=True)
        ge = torch.tensor(0.1, requires_grad=True)
        sc = ag.embedding_alignment_score(a, b, lengths, go, ge, locality, normalize=False)
        sc.sum().backward()
        Eb, Fb = Es.to(torch.bfloat16).float(), Et.to(torch.bfloat16).float()
        # the same BF16 tensor-core product (FP32 accumulation) as the fused forward
        St0 = torch.zeros((B, nt, ns), dtype=torch.float32, device="cuda")
        S = ag.similarity_bf16(Es.to(torch.bfloat16), Et.to(torch.bfloat16), lengths, out=St0)
        S = S.contiguous().requires_grad_(True)
        go2 = torch.tensor(0.5, requires_grad=True)
        ge2 = torch.tensor(0.1, requires_grad=True)
        sc2 = ag.alignment_score(S, lengths, go2, ge2, locality)
        sc2.sum().backward()
        assert torch.equal(sc, sc2)
        dS = S.grad.double()
        assert torch.allclose(a.grad.double(), torch.bmm(dS, Fb.double()), atol=1e-6)
        assert torch.allclose(b.grad.double(), torch.bmm(dS.transpose(1, 2), Eb.double()), atol=1e-6)
        assert abs(go.grad.item() - go2.grad.item()) < 1e-4 and abs(ge.grad.item() - ge2.grad.item()) < 1e-4


def test_fused_series_dtw_gradients_match_dense_route(torch_ag):
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(3)
    B, ns, nt = 16, 70, 90
    x0 = torch.cumsum(torch.randn(B, ns, device="cuda", generator=g), 1)
    y0 = torch.cumsum(torch.randn(B, nt, device="cuda", generator=g), 1)
    rng = np.random.default_rng(8)
    lengths = np.stack([rng.integers(1, ns + 1, B), rng.integers(1, nt + 1, B)], axis=1)
    x = x0.clone().requires_grad_(True)
    y = y0.clone().requires_grad_(True)
    sc = ag.dtw_series_score(x, y, lengths)
    sc.sum().backward()
    x2 = x0.clone().requires_grad_(True)
    y2 = y0.clone().requires_grad_(True)
    D = (x2[:, :, None] - y2[:, None, :]).abs()
    sc2 = ag.alignment_score(D, lengths, locality="global", direction="minimize", dtw=True)
    sc2.sum().backward()
    assert torch.equal(sc, sc2)
    assert torch.allclose(x.grad, x2.grad, atol=1e-5) and torch.allclose(y.grad, y2.grad, atol=1e-5)


def test_fused_cosine_gradients_match_torch_normalize(torch_ag):
    """With normalize=True the fused backward equals torch's autograd through F.normalize
    applied to dS @ en_t (the dense route), to float32 rounding."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(21)
    B, ns, nt, d = 16, 40, 36, 128
    Es = torch.randn(B, ns, d, device="cuda", generator=g)
    Et = torch.randn(B, nt, d, device="cuda", generator=g)
    lengths = np.full((B, 2), (ns, nt))
    a = Es.clone().requires_grad_(True)
    b = Et.clone().requires_grad_(True)
    sc = ag.embedding_alignment_score(a, b, lengths, 0.5, 0.1, "global", normalize=True)
    sc.sum().backward()
    a2 = Es.clone().requires_grad_(True)
    b2 = Et.clone().requires_grad_(True)
    en_s = torch.nn.functional.normalize(a2, dim=-1)
    en_t = torch.nn.functional.normalize(b2, dim=-1)
    # the float32 product of the BF16 factors (the tensor-core kernel keeps FP32 outputs)
    S = torch.bmm(en_t.to(torch.bfloat16).float(), en_s.to(torch.bfloat16).float().transpose(1, 2)).transpose(1, 2)
    sc2 = ag.alignment_score(S, lengths, 0.5, 0.1, "global")
    sc2.sum().backward()
    assert torch.allclose(sc, sc2, atol=1e-4)
    assert torch.allclose(a.grad, a2.grad, atol=2e-3, rtol=1e-2)
    assert torch.allclose(b.grad, b2.grad, atol=2e-3, rtol=1e-2)


@pytest.mark.parametrize("case", [("dtw", "global", "minimize"), ("affine", "global", "minimize"),
                                  ("linear", "local", "maximize")])
def test_series_paths_equal_dense_paths(torch_ag, case):
    """The series form (S = |x_u - y_v| computed in the kernel) gives the scores and paths of
    the dense form on the materialised matrix, bit for bit; the series rows are strided views
    of wider buffers, the lengths ragged down to one cell."""
    torch, ag = torch_ag
    kind, locality, direction = case
    g = torch.Generator(device="cuda").manual_seed(41)
    B, ns, nt = 40, 300, 257
    xb = torch.cumsum(torch.randn(B, ns + 20, device="cuda", generator=g), 1)
    yb = torch.cumsum(torch.randn(B, nt + 7, device="cuda", generator=g), 1)
    x, y = xb[:, 3:3 + ns], yb[:, 5:5 + nt]
    rng = np.random.default_rng(12)
    lengths = np.stack([rng.integers(1, ns + 1, B), rng.integers(1, nt + 1, B)], axis=1)
    lengths[0] = (1, 1)
    lengths[1] = (ns, nt)
    lengths[2] = (1, nt)
    dtw = kind == "dtw"
    gap = None if dtw else ((0.7, None) if kind == "linear" else (1.5, 0.4))
    s1, p1, l1, o1 = ag._series_paths(x, y, lengths, gap, locality, direction, dtw)
    D = (x[:, :, None] - y[:, None, :]).abs()
    s2, p2, l2, o2, _ = ag._forward_paths(D, lengths, gap, locality, direction, dtw)
    assert torch.equal(s1, s2)
    assert torch.equal(l1, l2) and torch.equal(o1, o2)
    o = o1.cpu().numpy()
    n = l1.cpu().numpy()
    P1, P2 = p1.cpu().numpy(), p2.cpu().numpy()
    for k in range(B):
        assert np.array_equal(P1[o[k]:o[k] + 2 * n[k]], P2[o[k]:o[k] + 2 * n[k]]), k


def test_series_dtw_weighted_gradients_match_path_counts(torch_ag):
    """The series backward with per-pair weights: dx_u = w_k * (number of the path's cells in
    row u with x_u > y_v minus those with x_u < y_v), dy likewise with the sign reversed --
    recomputed on the host from the forward's own paths (long paths: several warp steps)."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(9)
    B, ns, nt = 24, 400, 333
    x0 = torch.cumsum(torch.randn(B, ns, device="cuda", generator=g), 1)
    y0 = torch.cumsum(torch.randn(B, nt, device="cuda", generator=g), 1)
    rng = np.random.default_rng(4)
    lengths = np.stack([rng.integers(1, ns + 1, B), rng.integers(1, nt + 1, B)], axis=1)
    w = torch.randn(B, device="cuda", generator=g)
    x = x0.clone().requires_grad_(True)
    y = y0.clone().requires_grad_(True)
    (ag.dtw_series_score(x, y, lengths) * w).sum().backward()
    _, paths, plen, poff = ag._series_paths(x0, y0, lengths, None, "global", "minimize", True)
    P, n, o = paths.cpu().numpy(), plen.cpu().numpy(), poff.cpu().numpy()
    xs, ys, wk = x0.cpu().numpy(), y0.cpu().numpy(), w.cpu().numpy().astype(np.float64)
    dx = np.zeros((B, ns))
    dy = np.zeros((B, nt))
    for k in range(B):
        pts = P[o[k]:o[k] + 2 * n[k]].reshape(-1, 2)
        pts = pts[(pts[:, 0] >= 0) & (pts[:, 1] >= 0)]
        assert pts[0].tolist() == [lengths[k, 0] - 1, lengths[k, 1] - 1] and pts[-1].tolist() == [0, 0]
        sg = np.sign(xs[k, pts[:, 0]] - ys[k, pts[:, 1]]).astype(np.float64)
        np.add.at(dx[k], pts[:, 0], wk[k] * sg)
        np.add.at(dy[k], pts[:, 1], -wk[k] * sg)
    assert np.allclose(x.grad.cpu().numpy(), dx, rtol=1e-6, atol=1e-6)
    assert np.allclose(y.grad.cpu().numpy(), dy, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("dim", [16, 100, 128, 256, 384, 512, 520])
def test_normalized_bf16_rows_with_lengths(torch_ag, dim):
    """The length-aware BF16 factor: rows inside each pair's length are E / |E| rounded to
    BF16 (the row-wise kernel for widths that are multiples of 4 up to 512, the one-row kernel
    otherwise) and agree with the plain kernel's rows to one BF16 rounding step (it sums the
    squares in another order); rows past the length are zero with 1/|E| = 0; a row count that
    is not a multiple of the rows a warp takes."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(dim)
    B, n = 7, 37
    E = torch.randn(B, n, dim, device="cuda", generator=g)
    ln = np.array([0, 1, 5, 36, 37, 20, 3])
    Eb, inv = ag.normalized_bf16(E, True, ln)
    Eb0, inv0 = ag.normalized_bf16(E, True, None)
    d = Eb.shape[-1]
    Eb, Eb0 = Eb.view(B, n, d), Eb0.view(B, n, d)
    inv, inv0 = inv.view(B, n), inv0.view(B, n)
    ref = torch.nn.functional.normalize(E, dim=-1)
    for k in range(B):
        m = int(ln[k])
        assert torch.equal(Eb[k, m:], torch.zeros_like(Eb[k, m:])) and torch.equal(inv[k, m:], torch.zeros_like(inv[k, m:]))
        if m:
            # the same rounding of the same values; the plain kernel sums in another order
            assert torch.allclose(inv[k, :m], inv0[k, :m], rtol=1e-6)
            assert torch.allclose(Eb[k, :m, :dim].float(), ref[k, :m], atol=1e-2, rtol=1e-2)
            assert (Eb[k, :m].float() - Eb0[k, :m].float()).abs().max().item() <= 2 ** -8


def test_normalized_bf16_tiled_writes_only_the_product_tiles(torch_ag):
    """The tiled factor equals the length-aware one on every row below each length rounded up
    to the product's tile and leaves the rows beyond untouched; the product and the scores of
    the embedding form are unchanged."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(77)
    B, n, d = 6, 300, 128
    E = torch.randn(B, n, d, device="cuda", generator=g)
    ln = np.array([0, 1, 127, 128, 129, 300])
    full, inv_full = ag.normalized_bf16(E, True, ln)
    tiled, inv_t = ag.normalized_bf16(E, True, ln, tiled=True)
    for k in range(B):
        top = min(n, -(-int(ln[k]) // ag.SIM_TILE) * ag.SIM_TILE)
        assert torch.equal(tiled[k, :top], full[k, :top])
        assert torch.equal(inv_t.view(B, n)[k, :top], inv_full.view(B, n)[k, :top])
    lengths = np.stack([np.array([5, 64, 128, 200, 256, 256]), np.array([7, 100, 130, 256, 1, 256])], axis=1)
    Es = torch.randn(B, 256, d, device="cuda", generator=g)
    Et = torch.randn(B, 256, d, device="cuda", generator=g)
    a = ag.embedding_alignment_score(Es, Et, lengths, 0.5, 0.1, "global")
    Esb, _ = ag.normalized_bf16(Es, True, lengths[:, 0])
    Etb, _ = ag.normalized_bf16(Et, True, lengths[:, 1])
    S = ag.similarity_bf16(Esb, Etb, lengths)
    b = ag.alignment_score(S, lengths, 0.5, 0.1, "global")
    assert torch.equal(a, b)


@pytest.mark.parametrize("dim", [128, 48])
def test_embedding_gradients_full_writes_every_row(torch_ag, dim):
    """pa_path_embedding_gradients_full on NaN-filled outputs equals the accumulate-into-zeros
    entry bit for bit: every row is written (aligned rows with their gradient, the others --
    gap and padding rows -- with zeros).  dim 48: the one-row kernel after a memset."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(dim + 1)
    B, n = 12, 90
    Es = torch.randn(B, n, dim, device="cuda", generator=g)
    Et = torch.randn(B, n, dim, device="cuda", generator=g)
    rng = np.random.default_rng(dim)
    lengths = np.stack([rng.integers(1, n + 1, B), rng.integers(1, n + 1, B)], axis=1)
    lengths[0] = (n, n)
    Esb, inv_s = ag.normalized_bf16(Es, True, lengths[:, 0])
    Etb, inv_t = ag.normalized_bf16(Et, True, lengths[:, 1])
    S = ag.similarity_bf16(Esb, Etb, lengths)
    _, paths, plen, poff, _ = ag._forward_paths(S, lengths, (0.5, 0.1), "global", "maximize", False)
    grad = torch.randn(B, device="cuda", generator=g)
    Es16, Et16 = ag._pad16(Es), ag._pad16(Et)
    d = Es16.shape[-1]
    out = {}
    for name, fill in (("pa_path_embedding_gradients", 0.0), ("pa_path_embedding_gradients_full", float("nan"))):
        dEs = torch.full_like(Es16, fill)
        dEt = torch.full_like(Et16, fill)
        ag._alg.check(getattr(ag._lib(), name)(
            B, d, 1, paths.data_ptr(), poff.data_ptr(), plen.data_ptr(), grad.data_ptr(), Es16.data_ptr(),
            Et16.data_ptr(), Esb.data_ptr(), Etb.data_ptr(), inv_s.data_ptr(), inv_t.data_ptr(), n, n,
            dEs.data_ptr(), dEt.data_ptr(), torch.cuda.current_stream().cuda_stream))
        out[fill == 0.0] = (dEs, dEt)
    assert torch.equal(out[True][0], out[False][0]) and torch.equal(out[True][1], out[False][1])
