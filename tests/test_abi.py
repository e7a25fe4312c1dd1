"""The C-ABI library builds, loads and exports every symbol of include/*.h (CPU only)."""

import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    inc = os.path.join(REPO, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(pa_[a-z0-9_]+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def libpath():
    from pyalign_gb300 import build
    return build.build()


def test_exports_every_declared_symbol(libpath):
    declared = _declared()
    assert len(declared) >= 40
    lib = ctypes.CDLL(libpath)
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_fails_loudly(libpath):
    """Without a GPU the solve must fail with PA_ERR_NO_DEVICE, never fall back to the CPU."""
    import numpy as np
    from pyalign_gb300 import algorithm as alg
    if alg.lib().pa_device_count() > 0:
        pytest.skip("a GPU is present")
    import types
    opts = alg.m16.create_options({
        "solver": alg.Type.ALIGNMENT, "direction": alg.Direction.MAXIMIZE, "batch": False,
        "return_dup": False, "locality": alg.Locality.GLOBAL,
        "codomain": types.SimpleNamespace(detail=alg.Detail.SCORE, count=alg.Count.ONE),
        "gap_cost": None})
    solver = alg.m16.create_solver(8, 8, opts)
    with pytest.raises(RuntimeError, match="no CUDA device"):
        solver.solve_binary_for_score(np.zeros((1, 4), np.uint32), np.zeros((1, 4), np.uint32), 1.0, -1.0,
                                      np.array([[4], [4]], np.uint16))


def test_length_limits_and_options(libpath):
    """Solver creation checks (solver.h:496-503) run on the host."""
    import types
    from pyalign_gb300 import algorithm as alg
    d = {"solver": alg.Type.ALIGNMENT, "direction": alg.Direction.MAXIMIZE, "batch": True,
         "return_dup": False, "locality": alg.Locality.LOCAL,
         "codomain": types.SimpleNamespace(detail=alg.Detail.ALIGNMENT, count=alg.Count.ONE),
         "gap_cost": None}
    with pytest.raises(RuntimeError, match="exceeds maximum supported sequence length"):
        alg.m16.create_solver(20000, 10, alg.m16.create_options(d))
    s = alg.m32.create_solver(20000, 10, alg.m32.create_options(d))
    assert s.batch_size == alg.DEFAULT_BATCH_SIZE
    d["batch"] = False
    assert alg.m16.create_solver(10, 10, alg.m16.create_options(d)).batch_size == 1


def test_differentiable_forms_refuse_host_tensors(libpath):
    """The autograd forms run on the GPU only: host tensors are refused with a ValueError
    before any work (no CPU fallback)."""
    torch = pytest.importorskip("torch")
    import numpy as np
    from pyalign_gb300 import autograd as ag
    lengths = np.array([[4, 5]])
    with pytest.raises(ValueError, match="CUDA"):
        ag.alignment_score(torch.zeros(1, 4, 5), lengths, 1.0, 0.5, "global")
    with pytest.raises(ValueError, match="CUDA"):
        ag.dtw_series_score(torch.zeros(1, 4), torch.zeros(1, 5), lengths)


def test_result_and_report_entries_check_arguments(libpath):
    """The result-side entry points refuse null or out-of-range arguments before touching a
    device: the device enumeration, the direct-maps solve, and the per-bucket width report."""
    from pyalign_gb300 import algorithm as alg
    L = alg.lib()
    counts = (ctypes.c_int32 * 4)()
    assert L.pa_result_first_alignments(None, 4, counts, None, None, None) == alg.PA_ERR_INVALID_ARGUMENT
    assert L.pa_solve_batch_result(None, None, None, None, None) == alg.PA_ERR_INVALID_ARGUMENT
    assert L.pa_solver_last_bucket_widths(None, None) == alg.PA_ERR_INVALID_ARGUMENT
    import types
    opts = alg.m16.create_options({
        "solver": alg.Type.ALIGNMENT, "direction": alg.Direction.MAXIMIZE, "batch": True, "batch_size": 4,
        "return_dup": False, "locality": alg.Locality.LOCAL,
        "codomain": types.SimpleNamespace(detail=alg.Detail.ALIGNMENT, count=alg.Count.ONE), "gap_cost": None})
    solver = alg.m16.create_solver(8, 8, opts)
    widths = (ctypes.c_int32 * 4)(7, 7, 7, 7)
    alg.check(L.pa_solver_last_bucket_widths(solver.handle, widths))
    assert list(widths) == [0, 0, 0, 0]  # no solve yet: one width, reported as zeros
