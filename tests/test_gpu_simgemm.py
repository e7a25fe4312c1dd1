"""The tensor-core similarity product (pa_similarity_bf16, tcgen05) against torch (needs a GPU).

The kernel multiplies BF16 factors with FP32 accumulation in tensor memory, so it matches
a float32 product of the same BF16 values up to the order of the float32 additions.  It
writes only the cells inside each pair's lengths: the tests fill the output with NaN first
and check that everything outside the lengths is still NaN (tile edges at 127/128/129,
empty pairs, K chunks of 128 plus a partial one).
"""

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


@pytest.mark.parametrize("kernel", ["pipelined", "plain"])
@pytest.mark.parametrize("dim", [16, 64, 128, 256, 272])
def test_similarity_matches_float32_product(torch_ag, monkeypatch, dim, kernel):
    """Both kernels: the pipelined one (TMA loads, warp-specialised, double-buffered TMEM),
    the default, and the plain one (PA_SIM_KERNEL=plain)."""
    torch, ag = torch_ag
    if kernel == "plain":
        monkeypatch.setenv("PA_SIM_KERNEL", "plain")
    g = torch.Generator(device="cuda").manual_seed(dim)
    B, ns, nt = 9, 300, 280
    Es = torch.randn(B, ns, dim, device="cuda", generator=g).to(torch.bfloat16)
    Et = torch.randn(B, nt, dim, device="cuda", generator=g).to(torch.bfloat16)
    lengths = np.array([[300, 280], [1, 1], [127, 128], [128, 129], [129, 127], [0, 50], [50, 0],
                        [257, 3], [5, 280]])
    out = torch.full((B, nt, ns), float("nan"), device="cuda")
    S = ag.similarity_bf16(Es, Et, lengths, out=out)
    want = torch.bmm(Es.float(), Et.float().transpose(1, 2))  # exact products, float32 sums
    assert ag.tensor_core_status() == 0
    for k, (ls, lt) in enumerate(lengths):
        got = S[k, :ls, :lt]
        assert torch.isfinite(got).all(), k
        torch.testing.assert_close(got, want[k, :ls, :lt], rtol=1e-5, atol=2e-5 * np.sqrt(dim))
        inside = torch.zeros((ns, nt), dtype=torch.bool, device="cuda")
        inside[:ls, :lt] = True
        assert torch.isnan(S[k][~inside]).all(), f"pair {k}: written outside its lengths"


def test_similarity_many_pairs_ragged(torch_ag):
    """2048 pairs with lengths uniform in [1, 512] (several waves of persistent tiles)."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(7)
    rng = np.random.default_rng(7)
    B, n, dim = 2048, 512, 128
    lengths = rng.integers(1, n + 1, size=(B, 2))
    Es = torch.randn(B, n, dim, device="cuda", generator=g).to(torch.bfloat16)
    Et = torch.randn(B, n, dim, device="cuda", generator=g).to(torch.bfloat16)
    S = ag.similarity_bf16(Es, Et, lengths, out=torch.zeros((B, n, n), device="cuda"))
    want = torch.bmm(Es.float(), Et.float().transpose(1, 2))
    mask = (torch.arange(n, device="cuda")[None, :, None] < torch.as_tensor(lengths[:, 0], device="cuda")[:, None, None]) & \
           (torch.arange(n, device="cuda")[None, None, :] < torch.as_tensor(lengths[:, 1], device="cuda")[:, None, None])
    assert ag.tensor_core_status() == 0
    diff = (S - want).abs()[mask]
    assert float(diff.max()) <= 1e-5 * float(want.abs()[mask].max()) + 1e-4
    assert float(S[~mask].abs().max()) == 0.0


def test_cosine_similarity_backward_matches_torch(torch_ag):
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(11)
    Es = torch.randn(6, 40, 48, device="cuda", generator=g)   # d = 48: padded to 48 (16 | 48)
    Et = torch.randn(6, 30, 48, device="cuda", generator=g)
    W = torch.randn(6, 40, 30, device="cuda", generator=g)
    a = Es.clone().requires_grad_(True)
    b = Et.clone().requires_grad_(True)
    (ag.cosine_similarity_batch(a, b) * W).sum().backward()
    a2 = Es.clone().requires_grad_(True)
    b2 = Et.clone().requires_grad_(True)
    en_s = torch.nn.functional.normalize(a2, dim=-1)
    en_t = torch.nn.functional.normalize(b2, dim=-1)
    S2 = torch.bmm(en_s.to(torch.bfloat16).float(), en_t.to(torch.bfloat16).float().transpose(1, 2))
    (S2 * W).sum().backward()
    torch.testing.assert_close(a.grad, a2.grad, rtol=2e-2, atol=2e-3)
    torch.testing.assert_close(b.grad, b2.grad, rtol=2e-2, atol=2e-3)


def test_epilogue_distance(torch_ag):
    """alpha = -1, beta = 1: the kernel writes 1 - <x, y> (one rounding), and DTW on it
    scores like DTW on torch's 1 - S."""
    torch, ag = torch_ag
    g = torch.Generator(device="cuda").manual_seed(13)
    B, ns, nt, dim = 5, 200, 150, 64
    Es = torch.nn.functional.normalize(torch.randn(B, ns, dim, device="cuda", generator=g), dim=-1)
    Et = torch.nn.functional.normalize(torch.randn(B, nt, dim, device="cuda", generator=g), dim=-1)
    Esb, Etb = Es.to(torch.bfloat16), Et.to(torch.bfloat16)
    lengths = np.array([[200, 150], [17, 150], [200, 1], [128, 129], [64, 64]])
    S = ag.similarity_bf16(Esb, Etb, lengths, out=torch.zeros((B, nt, ns), device="cuda"))
    D = ag.similarity_bf16(Esb, Etb, lengths, out=torch.ones((B, nt, ns), device="cuda"), alpha=-1.0, beta=1.0)
    assert ag.tensor_core_status() == 0
    for k, (ls, lt) in enumerate(lengths):
        assert torch.equal(D[k, :ls, :lt], 1.0 - S[k, :ls, :lt]), k
    a = ag.alignment_score(D, lengths, locality="global", direction="minimize", dtw=True)
    b = ag.alignment_score((1.0 - S).contiguous(), lengths, locality="global", direction="minimize", dtw=True)
    assert torch.equal(a, b), (a, b)
