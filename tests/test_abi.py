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


_LAYOUT_C = r"""
#include <stdio.h>
#include "pyalign_gb300.h"
#define F(T, f) printf("%s.%s %zu %zu\n", #T, #f, offsetof(T, f), sizeof(((T *)0)->f));
#define C(x) printf("%s %ld\n", #x, (long)(x));
int main(void) {
	printf("pa_options %zu\npa_batch %zu\n", sizeof(pa_options), sizeof(pa_batch));
	F(pa_options, type) F(pa_options, direction) F(pa_options, detail) F(pa_options, count)
	F(pa_options, locality) F(pa_options, remove_dup) F(pa_options, batch) F(pa_options, batch_size)
	F(pa_options, index_bits) F(pa_options, gap_kind) F(pa_options, linear_s) F(pa_options, linear_t)
	F(pa_options, affine_u_s) F(pa_options, affine_v_s) F(pa_options, affine_u_t) F(pa_options, affine_v_t)
	F(pa_options, general_s) F(pa_options, general_t)
	F(pa_batch, form) F(pa_batch, location) F(pa_batch, batch) F(pa_batch, n_s) F(pa_batch, n_t)
	F(pa_batch, a) F(pa_batch, b) F(pa_batch, sim) F(pa_batch, table) F(pa_batch, table_rows)
	F(pa_batch, table_cols) F(pa_batch, eq) F(pa_batch, ne) F(pa_batch, length)
	C(PA_OK) C(PA_ERR_INVALID_ARGUMENT) C(PA_ERR_LENGTH) C(PA_ERR_UNSUPPORTED)
	C(PA_TYPE_ALIGNMENT) C(PA_TYPE_DTW) C(PA_MINIMIZE) C(PA_MAXIMIZE)
	C(PA_DETAIL_SCORE) C(PA_DETAIL_ALIGNMENT) C(PA_DETAIL_SOLUTION) C(PA_COUNT_ONE) C(PA_COUNT_ALL)
	C(PA_LOCAL) C(PA_GLOBAL) C(PA_SEMIGLOBAL)
	return 0;
}
"""


def test_python_binding_matches_the_header_layout(tmp_path):
    """The ctypes structures and constants of the Python binding are the header's: a C
    program compiled against include/pyalign_gb300.h prints every field's offset and size of
    pa_options and pa_batch and the enum values, and the binding must agree with each (a
    drifted field would pass garbage through the C ABI without any error)."""
    import shutil
    import subprocess
    from pyalign_gb300 import algorithm as alg
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text(_LAYOUT_C)
    subprocess.run([cc, "-std=c11", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c = {}
    for line in filter(None, out):
        k, *v = line.split()
        c[k] = tuple(int(x) for x in v) if len(v) > 1 else int(v[0])
    for name, cls in (("pa_options", alg._Options), ("pa_batch", alg.Batch)):
        assert ctypes.sizeof(cls) == c[name], name
        fields = [f[0] for f in cls._fields_]
        assert fields == [k.split(".", 1)[1] for k in c if k.startswith(name + ".")], name
        for f in fields:
            desc = getattr(cls, f)
            assert (desc.offset, desc.size) == c[f"{name}.{f}"], (name, f)
    assert (alg.PA_OK, alg.PA_ERR_INVALID_ARGUMENT, alg.PA_ERR_LENGTH, alg.PA_ERR_UNSUPPORTED) == (
        c["PA_OK"], c["PA_ERR_INVALID_ARGUMENT"], c["PA_ERR_LENGTH"], c["PA_ERR_UNSUPPORTED"])
    assert (alg.Type.ALIGNMENT, alg.Type.DTW) == (c["PA_TYPE_ALIGNMENT"], c["PA_TYPE_DTW"])
    assert (alg.Direction.MINIMIZE, alg.Direction.MAXIMIZE) == (c["PA_MINIMIZE"], c["PA_MAXIMIZE"])
    assert (alg.Detail.SCORE, alg.Detail.ALIGNMENT, alg.Detail.SOLUTION) == (
        c["PA_DETAIL_SCORE"], c["PA_DETAIL_ALIGNMENT"], c["PA_DETAIL_SOLUTION"])
    assert (alg.Count.ONE, alg.Count.ALL) == (c["PA_COUNT_ONE"], c["PA_COUNT_ALL"])
    assert (alg.Locality.LOCAL, alg.Locality.GLOBAL, alg.Locality.SEMIGLOBAL) == (
        c["PA_LOCAL"], c["PA_GLOBAL"], c["PA_SEMIGLOBAL"])


def _prototypes():
    """{name: (return type, [parameter types])} of every function include/*.h declares, each
    type reduced to 'ptr' or its fixed-width scalar name."""
    scal = {"int64_t": "i64", "int32_t": "i32", "uint32_t": "u32", "uint64_t": "u64", "float": "f32",
            "double": "f64", "pa_status": "i32", "void": "void"}

    def kind(decl):
        decl = decl.strip()
        if "*" in decl:
            return "ptr"
        words = [w for w in re.findall(r"[A-Za-z_][A-Za-z0-9_]*", decl) if w not in ("const", "struct")]
        return scal[words[0]]

    protos = {}
    inc = os.path.join(REPO, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        src = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
        src = re.sub(r"^\s*#.*$", "", src, flags=re.M)
        for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(pa_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src):
            ret, name, params = m.group(1), m.group(2), m.group(3).strip()
            args = [] if params in ("", "void") else [kind(p) for p in params.split(",")]
            protos[name] = (kind(ret + (" *" if ret.rstrip().endswith("*") else "")), args)
    return protos


def test_ctypes_prototypes_match_the_header(libpath):
    """Every argtypes/restype the package's bindings give a C function (algorithm.py,
    prepare.py, autograd.py) agrees with its declaration in include/*.h, parameter by
    parameter: a pointer where the header has a pointer, the same fixed-width scalar
    elsewhere, and a return type that does not truncate (int64 results, float, strings)."""
    pytest.importorskip("torch")
    from pyalign_gb300 import algorithm as alg
    from pyalign_gb300 import autograd as ag
    from pyalign_gb300 import prepare
    L = alg.lib()
    prepare._lib()
    ag._lib()
    protos = _prototypes()
    assert len(protos) == len(_declared())

    def kind(t):
        if t is None:
            return "i32"     # ctypes' default int return
        if t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, ctypes._Pointer):
            return "ptr"
        return {ctypes.c_int64: "i64", ctypes.c_int32: "i32", ctypes.c_uint32: "u32",
                ctypes.c_uint64: "u64", ctypes.c_float: "f32", ctypes.c_double: "f64"}[t]

    checked = 0
    for name, (ret, args) in sorted(protos.items()):
        fn = getattr(L, name)
        at = getattr(fn, "argtypes", None)
        if at is None and args:
            continue         # not bound by the package (diagnostics, the allocation-free entry)
        assert [kind(t) for t in (at or [])] == args, name
        if ret != "void":
            assert kind(fn.restype) == ret, (name, ret)
        checked += 1
    assert checked >= 55
