"""The C ABI library loads and exports every function the public headers declare.

No compute call is made by the CPU tests here; create-type calls are only
checked for their error status when no device is visible.  The one GPU test
runs the compiled C++ drop-in caller.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for mt in re.finditer(r"\b((?:gpunmf|gpumlib)_\w+)\s*\(", text):
            names.append(mt.group(1))
    return sorted(set(names))


def test_headers_declare_functions():
    names = declared_functions()
    assert "gpunmf_create" in names and "gpumlib_cuda_nmf_multiplicative_euclidean_update_matrix" in names


def test_library_exports_every_declared_symbol(built):
    from gpumlib_gb300 import _native
    lib = _native.load()
    out = subprocess.run(["nm", "-D", "--defined-only", _native.lib_path()], capture_output=True, text=True)
    exported = set(l.split()[-1] for l in out.stdout.splitlines() if l.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, "declared but not exported: %s" % missing
    bound = set(s[0] for s in _native.SIGNATURES)
    unbound = [n for n in declared_functions() if n not in bound]
    assert not unbound, "declared but without a ctypes signature: %s" % unbound
    for n in declared_functions():
        getattr(lib, n)


def test_version_and_host_only_calls(built):
    from gpumlib_gb300 import _native, inputs
    lib = _native.load()
    assert b"sm_103a" in lib.gpunmf_version()
    out = np.empty(1000, dtype=np.float32)
    lib.gpunmf_fill_uniform(7, 123, out.size, out.ctypes.data_as(ctypes.c_void_p))
    assert np.array_equal(out, inputs.uniform(7, 1000, offset=123))
    assert lib.gpunmf_footprint_bytes(0, 8192, 8192, 64, 0) > 8192 * 8192 * 4
    assert lib.gpunmf_footprint_bytes(0, 0, 10, 2, 0) == 0


def test_null_handle_errors(built):
    from gpumlib_gb300 import _native
    lib = _native.load()
    assert lib.gpunmf_iterate(None, 1, 1) == 1
    assert lib.gpunmf_destroy(None) == 1
    assert b"null" in lib.gpunmf_last_error()


def test_create_without_gpu_reports_no_device(built):
    from gpumlib_gb300 import _native
    lib = _native.load()
    if lib.gpunmf_device_count() > 0:
        pytest.skip("a GPU is visible")
    V = np.ones((4, 3), dtype=np.float32, order="F")
    W = np.ones((4, 2), dtype=np.float32, order="F")
    H = np.ones((2, 3), dtype=np.float32, order="F")
    h = ctypes.c_void_p()
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    st = lib.gpunmf_create(0, 4, 3, 2, p(V), p(W), p(H), 1e-8, 0, None, ctypes.byref(h))
    assert st == 5  # GPUNMF_ERR_NO_DEVICE
    assert st == lib.gpunmf_create(0, 4, 3, 2, p(V), p(W), p(H), 1e-8, 0, None, ctypes.byref(h))


def test_invalid_arguments_rejected_before_device(built):
    from gpumlib_gb300 import _native
    lib = _native.load()
    h = ctypes.c_void_p()
    V = np.ones((4, 3), dtype=np.float32, order="F")
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.gpunmf_create(9, 4, 3, 2, p(V), p(V), p(V), 1e-8, 0, None, ctypes.byref(h)) == 1
    assert lib.gpunmf_create(0, 4, 3, 0, p(V), p(V), p(V), 1e-8, 0, None, ctypes.byref(h)) == 1
    assert lib.gpunmf_create(0, 4, 3, 2, None, p(V), p(V), 1e-8, 0, None, ctypes.byref(h)) == 1
    assert lib.gpunmf_create(0, 4, 3, 2, p(V), p(V), p(V), -1.0, 0, None, ctypes.byref(h)) == 1
    assert lib.gpunmf_create(0, 4, 3, 2, p(V), p(V), p(V), 1e-8, 7, None, ctypes.byref(h)) == 1


def test_cpp_dropin_header_compiles(built, tmp_path):
    """A FacesNMF-style caller compiles against include/gpumlib_nmf.hpp and links the library."""
    from gpumlib_gb300 import _native
    src = tmp_path / "caller.cpp"
    src.write_text(CPP_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_native.lib_path())
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-I", os.path.join(ROOT, "include"), "-I", cuda + "/include",
                        str(src), "-o", str(exe), "-L", libdir, "-lgpunmf", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_dropin_caller_runs(built, tmp_path):
    """The same caller runs on the GPU; the reference-form additive Euclidean class leaves H as given."""
    from gpumlib_gb300 import _native
    src = tmp_path / "caller.cpp"
    src.write_text(CPP_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_native.lib_path())
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-I", os.path.join(ROOT, "include"), "-I", cuda + "/include",
                        str(src), "-o", str(exe), "-L", libdir, "-lgpunmf", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    lines = run.stdout.split("\n")
    ae_h, ae2_h, ad_w = (float(x) for x in lines[2].split())
    assert ae_h == np.float32(0.5), "fixed-H additive class changed H"
    assert ae2_h != np.float32(0.5) and ae2_h >= 0 and ad_w >= 0


CPP_CALLER = r"""
#include <cstdio>
#include "gpumlib_nmf.hpp"
using namespace GPUMLib;
int main() {
    int n = 40, m = 30, r = 4;
    HostMatrix<cudafloat> V(n, m, ColumnMajor), W(n, r, ColumnMajor), H(r, m, ColumnMajor);
    for (int j = 0; j < m; j++) for (int i = 0; i < n; i++) V(i, j) = (float)((i * 7 + j * 3) % 11) / 11.0f;
    for (int a = 0; a < r; a++) for (int i = 0; i < n; i++) W(i, a) = 0.5f + 0.01f * ((i + a) % 5);
    for (int j = 0; j < m; j++) for (int a = 0; a < r; a++) H(a, j) = 0.5f + 0.01f * ((j + a) % 7);
    try {
        NMF_MultiplicativeEuclidianDistance nmf(V, W, H);
        NMF * p = &nmf;
        for (int it = 0; it < 50; it++) { p->DoIteration(); if (p->QualityImprovement() < 0.0001f) break; }
        HostMatrix<cudafloat> w = p->GetW(), h = p->GetH(), wh = p->GetWH();
        std::printf("%.9g %.9g %.9g %.12g\n", w(0, 0), h(0, 0), wh(0, 0), nmf.Residual());
        NMF_MultiplicativeDivergence kl(V, W, H);
        kl.DoIteration(true); kl.DoIteration(false);
        HostMatrix<cudafloat> kw = kl.GetW();
        std::printf("%.9g %.12g\n", kw(1, 1), kl.ObjectiveKL());
        NMF_AdditiveEuclidian ae(V, W, H);          // the reference GPU class: H stays as given
        NMF_AdditiveEuclidian ae2(V, W, H, true);   // H updated as well
        NMF_AdditiveDivergence ad(V, W, H);
        ae.DoIteration(); ae2.DoIteration(); ad.DoIteration();
        std::printf("%.9g %.9g %.9g\n", ae.GetH()(0, 0), ae2.GetH()(0, 0), ad.GetW()(0, 0));
    } catch (NMFError & e) {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return 2;
    }
    return 0;
}
"""


def header_prototypes():
    """{name: (return type, [parameter types])} of every function include/gpunmf.h declares."""
    text = open(os.path.join(ROOT, "include", "gpunmf.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, params in re.findall(r"\b([A-Za-z_][\w ]*?\**)\s*\b((?:gpunmf|gpumlib)_\w+)\s*\(([^;{]*?)\)\s*;",
                                        text, flags=re.S):
        ps = [] if params.strip() in ("", "void") else [re.sub(r"\s+", " ", p.strip()) for p in params.split(",")]
        # drop the parameter name, keep the type
        types = [re.sub(r"\s*\b\w+$", "", p) if not p.endswith("*") else p for p in ps]
        ret = re.sub(r"^(?:extern\s+\"C\"\s+|GPUNMF_API\s+)", "", ret.strip())
        out[name] = (ret.strip(), types)
    return out


def _kind_of_c(t):
    """Canonical kind of a C type: 'ptr', 'dim3', 'void', or (class, bytes, signed)."""
    t = t.replace("const ", "").strip()
    if "*" in t or t in ("gpunmf_handle",):
        return "ptr"
    size_t = ctypes.sizeof(ctypes.c_size_t)
    return {"int": ("int", 4, True), "unsigned int": ("int", 4, False), "unsigned": ("int", 4, False),
            "long long": ("int", 8, True), "unsigned long long": ("int", 8, False), "size_t": ("int", size_t, False),
            "float": ("float", 4, True), "double": ("float", 8, True), "gpunmf_dim3": "dim3", "void": "void",
            # the header's enums are passed and returned as int
            "gpunmf_status": ("int", 4, True), "gpunmf_rule": ("int", 4, True),
            "gpunmf_precision": ("int", 4, True)}[t]


def _kind_of_ctypes(c):
    from gpumlib_gb300 import _native
    if c is None:
        return "void"
    if c in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(c, ctypes._Pointer):
        return "ptr"
    if c is _native.Dim3:
        return "dim3"
    code = c._type_
    if code in "fd":
        return ("float", ctypes.sizeof(c), True)
    return ("int", ctypes.sizeof(c), code.islower())


def test_ctypes_signatures_match_header():
    """Every header function has a ctypes signature with the same arity, argument kinds and return kind."""
    from gpumlib_gb300 import _native
    protos = header_prototypes()
    assert len(protos) >= 50
    sigs = {name: (res, args) for name, res, args in _native.SIGNATURES}
    assert sorted(protos) == sorted(sigs), set(protos) ^ set(sigs)
    for name, (ret, params) in protos.items():
        res, args = sigs[name]
        assert len(args) == len(params), (name, params, args)
        for k, (p, a) in enumerate(zip(params, args)):
            assert _kind_of_c(p) == _kind_of_ctypes(a), (name, k, p, a)
        assert _kind_of_c(ret) == _kind_of_ctypes(res), (name, ret, res)


def test_python_constants_match_header_macros():
    """The Python mirror's constants are the header's values (the quality sampling mode, the rules,
    the precisions)."""
    import gpumlib_gb300 as g
    text = open(os.path.join(ROOT, "include", "gpunmf.h")).read()
    mt = re.search(r"#define\s+GPUNMF_QUALITY_WHEN_READY\s+\((-?\d+)\)", text)
    assert mt and int(mt.group(1)) == g.QUALITY_WHEN_READY
    values = {name: int(v) for name, v in re.findall(r"\b(GPUNMF_\w+)\s*=\s*(-?\d+)", text)}
    assert values.get("GPUNMF_EUCLIDEAN") == g.EUCLIDEAN and values.get("GPUNMF_DIVERGENCE") == g.DIVERGENCE
    assert values.get("GPUNMF_FP32") == g.nmf.PRECISIONS["fp32"] and values.get("GPUNMF_BF16") == g.nmf.PRECISIONS["bf16"]
