"""Device path of the batch encoder (needs a GPU): one upload of the raw bytes, a kernel
maps them through the alphabet's index into device code rows; the rows equal the host
path's, a byte outside the alphabet raises, and the device codes solve like host codes."""

import numpy as np
import pytest

from _cases import Gap, compare, options

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from pyalign_gb300 import build
    build.build()
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device visible")
    from pyalign_gb300 import algorithm as alg
    from pyalign_gb300 import prepare as prep
    return torch, alg, prep


def _strings(rng, n, lo, hi):
    return ["".join(rng.choice(list("ACGT"), size=int(rng.integers(lo, hi + 1)))) for _ in range(n)]


def test_device_encoding_equals_host(env):
    torch, alg, prep = env
    rng = np.random.default_rng(8)
    strings = _strings(rng, 5000, 0, 700)
    lut = prep.lut_of("GATC")
    host, lens = prep.encode_latin1(strings, lut, width=700)
    dev = torch.full((5000, 704), -1, dtype=torch.int32, device="cuda")
    prep.encode_latin1(strings, lut, out=dev, width=700)
    got = dev.cpu().numpy().view(np.uint32)
    assert np.array_equal(got[:, :700], host)
    assert (got[:, 700:] == 0xFFFFFFFF).all()  # beyond width: untouched
    with pytest.raises(ValueError, match="item not in alphabet"):
        prep.encode_latin1(strings[:10] + ["ACGX"], lut, out=dev, width=700)


def test_device_codes_solve_like_host_codes(env, oracle_alg):
    import ctypes
    torch, alg, prep = env
    rng = np.random.default_rng(9)
    n = 777
    s_list, t_list = _strings(rng, n, 1, 300), _strings(rng, n, 1, 320)
    lut = prep.lut_of("ACGT")
    a_d = torch.zeros((n, 300), dtype=torch.int32, device="cuda")
    b_d = torch.zeros((n, 320), dtype=torch.int32, device="cuda")
    prep.encode_latin1(s_list, lut, out=a_d)
    prep.encode_latin1(t_list, lut, out=b_d)
    a_h, _ = prep.encode_latin1(s_list, lut, width=300)
    b_h, _ = prep.encode_latin1(t_list, lut, width=320)
    table = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(table, 2.0)
    t_d = torch.from_numpy(table).cuda()
    ln = np.stack([[len(s) for s in s_list], [len(t) for t in t_list]]).astype(np.int32)
    opts = dict(options(alg, locality="local", detail="alignment", gap=Gap("affine", 5.0, 2.0)), batch_size=n)
    solver = alg.m16.create_solver(300, 320, alg.m16.create_options(opts))
    alg.check(alg.lib().pa_solver_set_stream(solver.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    P = ctypes.POINTER
    sizes = np.minimum(ln[0], ln[1]).astype(np.int64)
    offs = np.zeros(n, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    sc = torch.empty(n, device="cuda")
    mp = torch.empty(int(sizes.sum()), dtype=torch.int32, device="cuda")
    bt = alg.Batch(form=1, location=1, batch=n, n_s=300, n_t=320, a=ctypes.cast(a_d.data_ptr(), P(ctypes.c_uint32)),
                   b=ctypes.cast(b_d.data_ptr(), P(ctypes.c_uint32)), table=ctypes.cast(t_d.data_ptr(), P(ctypes.c_float)),
                   table_rows=4, table_cols=4, length=ln.ctypes.data_as(P(ctypes.c_int32)))
    alg.check(alg.lib().pa_solve_batch(solver.handle, ctypes.byref(bt), ctypes.c_void_p(sc.data_ptr()),
                                       ctypes.c_void_p(mp.data_ptr()), offs.ctypes.data_as(P(ctypes.c_int64))))
    torch.cuda.synchronize()
    oracle = oracle_alg.m16.create_solver(300, 320, oracle_alg.m16.create_options(opts))
    want = oracle.solve_indexed_for_alignment(a_h, b_h, table, ln.astype(np.uint16))
    scores = sc.cpu().numpy()
    maps = mp.cpu().numpy()
    for k in range(n):
        w = want[k]
        assert scores[k] == w.score, k
        s2t = maps[offs[k]:offs[k] + sizes[k]]
        ref = w.s_to_t if ln[0, k] <= ln[1, k] else w.t_to_s
        assert np.array_equal(s2t, ref), k
