"""C ABI checks that need no GPU: the library loads, exports every function
include/idrs_gb300.h declares, and rejects bad arguments before touching the
device."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "idrs_gb300.h")


def _declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|long|const char \*)\s*(idrs_\w+)\(", src, re.M)))


def test_library_exports_every_declared_symbol(pkg):
    lib_path = pkg.build_recipe.build()
    lib = C.CDLL(lib_path)
    names = _declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_prototypes_cover_the_header(pkg):
    assert set(_declared()) <= set(pkg.api._PROTOS)


def test_pp_structs_match_the_c_layout(pkg):
    """The ctypes mirrors of idrs_pp_options / _report / _inputs have the
    C structs' sizes (a field added on one side only changes them)."""
    lib = pkg.load()
    api = pkg.api
    for which, cls in enumerate((api.PPOptions, api.PPReport, api.PPInputs)):
        assert lib.idrs_pp_struct_size(which) == C.sizeof(cls), cls.__name__
    assert lib.idrs_pp_struct_size(3) == 0


def test_fp64_check_tolerance_rules(pkg):
    """fp64_check: None checks mixed results of host-array calls only, True
    any result at tol * 1e-3 (at least 1e-14), a float is the tolerance."""
    import pytest
    f = pkg.api.fp64_check_tolerance
    assert f(1e-8, None, True) == pytest.approx(1e-11)
    assert f(1e-8, None, False) == 0.0
    assert f(1e-8, None, True, dev=True) == 0.0
    assert f(1e-8, True, False, dev=True) == pytest.approx(1e-11)
    assert f(1e-13, True, True) == 1e-14
    assert f(1e-8, False, True) == 0.0
    assert f(1e-8, 3e-12, False) == 3e-12
    with pytest.raises(pkg.api.IDRSError):
        f(1e-8, -1.0, True)
    o = pkg.api._pp_options(0, 8, 1e-8, 60, 4, 300, 3e-3, 2, 8, 20, 32, False, 0, False, 1, None)
    assert o.fp64_check_tol == pytest.approx(1e-11) and o.poly_eval == 1
    o = pkg.api._pp_options(0, 8, 1e-8, 60, 4, 0, 3e-3, 2, 8, 20, 64, False, 0, False, 1, None)
    assert o.fp64_check_tol == 0.0


def test_argument_errors_without_gpu(pkg):
    lib = pkg.load()
    h = C.c_void_p()
    st = lib.idrs_crs_format(-1, 3, None, None, None, None, C.byref(h))
    assert st == pkg.api.IDRS_ERR_ARG
    assert b"crs_format" in lib.idrs_last_error()
    st = lib.idrs_stencil7_format(0, 3, 3, None, C.byref(h))
    assert st == pkg.api.IDRS_ERR_ARG
    assert lib.idrs_matrix_create(None, None, 0, None, C.byref(h)) == pkg.api.IDRS_ERR_ARG
    assert lib.idrs_version() >= 10000


def test_pp_idrs_host_output_buffer(pkg, monkeypatch):
    """PP_IDRS with a host b writes the solution into a caller's x_out (for
    example pinned memory) and rejects an unsuitable one; a fake library
    stands in for the device call."""
    import types
    import numpy as np
    import pytest
    api = pkg.api
    n = 7
    seen = {}

    def fake_pp(K, pb, P, c, f, inp, o, rep, px):
        seen["px"] = px
        (C.c_double * n).from_address(px)[:] = [float(i) for i in range(n)]
        return 0

    fake = types.SimpleNamespace(idrs_rpp_idrs_ext=fake_pp, idrs_last_error=lambda: b"")
    monkeypatch.setattr(api, "_lib", fake)
    K = types.SimpleNamespace(handle=None, nrows=n, cplx=False)
    b = np.ones(n)
    out = np.full(n, -1.0)
    r = api.PP_IDRS(K, b, x_out=out)
    assert r.x is out and seen["px"] == out.ctypes.data
    np.testing.assert_array_equal(out, np.arange(n, dtype=float))
    r = api.PP_IDRS(K, b)  # no x_out: a fresh array
    assert r.x is not out and seen["px"] == r.x.ctypes.data
    for bad in (np.zeros(n + 1), np.zeros(n, dtype=np.float32), np.zeros((n, 2))[:, 0], [0.0] * n):
        with pytest.raises(ValueError):
            api.PP_IDRS(K, b, x_out=bad)


def test_multishift_shift_masks(pkg):
    """The per-shift status a multishift result carries: a NaN residual or
    solution column is non-finite (never converged), the others converge by
    relres <= tol."""
    import numpy as np
    x = np.ones((4, 3))
    x[2, 1] = np.nan
    r = pkg.api.Result(x=x, relres=np.array([1e-9, 1e-9, np.nan]), flag=0, iterations=5)
    pkg.api._shift_masks(r, 1e-8)
    np.testing.assert_array_equal(r.nonfinite_mask, [False, True, True])
    np.testing.assert_array_equal(r.converged_mask, [True, False, False])
    r = pkg.api.Result(x=np.ones((4, 2)), relres=np.array([1e-7, 1e-9]), flag=2, iterations=5)
    pkg.api._shift_masks(r, 1e-8)
    np.testing.assert_array_equal(r.converged_mask, [False, True])
