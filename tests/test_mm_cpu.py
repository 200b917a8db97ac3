"""Matrix Market input (mm_matrix, E/MATRIX_MARKET/mm_module.f90:48-154):
the host conversion idrs_mm_read against scipy.io.mmread on files written
here, covering every representation, field and symmetry the reader accepts.
No GPU needed."""
import os

import numpy as np
import pytest

sio = pytest.importorskip("scipy.io")
pytestmark = pytest.mark.filterwarnings("ignore::DeprecationWarning")

# the reference's example files (E/MATRIX_MARKET/DATA), when a checkout of the
# reference is at hand: IDRS_REFERENCE_MM_DATA names that directory; the tests
# that read them are skipped without it
REF_DATA = os.environ.get("IDRS_REFERENCE_MM_DATA", "")


def _write(path, banner, size, lines):
    with open(path, "w") as f:
        f.write(banner + "\n% a comment\n%\n")
        f.write(size + "\n")
        for ln in lines:
            f.write(ln + "\n")
    return str(path)


def _dense_from(r, cplx):
    n, m = r.nrows, r.ncols
    D = np.zeros((n, m), dtype=np.complex128 if cplx else np.float64)
    if r.rep == "array":
        return r.vals
    if "row_ptr" in r:
        for i in range(n):
            for p in range(r.row_ptr[i] - 1, r.row_ptr[i + 1] - 1):
                D[i, r.col_ind[p] - 1] += r.vals[p] if r.field != "pattern" else 1.0
    else:
        for p in range(r.nnz):
            D[r.indx[p] - 1, r.jndx[p] - 1] += r.vals[p] if r.field != "pattern" else 1.0
    return D


def _scipy_dense(path, cplx):
    A = sio.mmread(path)
    A = A.toarray() if hasattr(A, "toarray") else np.asarray(A)
    if cplx:  # the reference's reader keeps complex entries in single precision
        A = A.astype(np.complex64).astype(np.complex128)
    return A


def _coords(rng, n, m, k, lower=False, strict=False):
    out = set()
    while len(out) < k:
        i, j = int(rng.integers(1, n + 1)), int(rng.integers(1, m + 1))
        if lower and (j > i or (strict and j == i)):
            continue
        out.add((i, j))
    return sorted(out, key=lambda t: (t[1], t[0]))


CASES = ["real general", "real symmetric", "real skew-symmetric", "complex general",
         "complex symmetric", "complex hermitian", "integer general", "integer symmetric",
         "pattern general", "pattern symmetric"]


@pytest.mark.parametrize("kind", CASES)
@pytest.mark.parametrize("fmt", [None, "coo", "crs"])
def test_coordinate_files_match_scipy(pkg, tmp_path, kind, fmt):
    field, symm = kind.split()
    rng = np.random.default_rng(hash(kind) % 2 ** 31)
    n = 23
    m = n if symm != "general" else 17
    lower = symm != "general"
    ij = _coords(rng, n, m, 60, lower=lower, strict=symm == "skew-symmetric")
    lines = []
    for i, j in ij:
        if field == "real":
            lines.append(f"{i} {j} {rng.standard_normal():.17e}")
        elif field == "complex":
            im = 0.0 if (symm == "hermitian" and i == j) else rng.standard_normal()
            lines.append(f"{i} {j} {rng.standard_normal():.17e} {im:.17e}")
        elif field == "integer":
            lines.append(f"{i} {j} {int(rng.integers(-9, 10))}")
        else:
            lines.append(f"{i} {j}")
    path = _write(tmp_path / "a.mtx", f"%%MatrixMarket matrix coordinate {field} {symm}",
                  f"{n} {m} {len(ij)}", lines)
    r = pkg.mm_read(path, fmt)
    assert (r.nrows, r.ncols, r.field, r.rep) == (n, m, field, "coordinate")
    mirrors = sum(1 for i, j in ij if i != j) if lower else 0
    assert r.nnz == len(ij) + mirrors
    cplx = field == "complex"
    np.testing.assert_array_equal(_dense_from(r, cplx), _scipy_dense(path, cplx))
    if fmt == "crs":  # rows keep the file order, each mirror right after its entry
        assert np.all(np.diff(r.row_ptr) >= 0) and r.row_ptr[0] == 1


@pytest.mark.parametrize("kind", ["real general", "real symmetric", "real skew-symmetric",
                                  "complex general", "complex hermitian", "integer general"])
def test_array_files_match_scipy(pkg, tmp_path, kind):
    field, symm = kind.split()
    rng = np.random.default_rng(7)
    n = 9
    m = n if symm != "general" else 4
    lines = []
    for j in range(m):
        r0 = 0 if symm == "general" else (j + 1 if symm == "skew-symmetric" else j)
        for i in range(r0, n):
            if field == "complex":
                im = 0.0 if (symm == "hermitian" and i == j) else rng.standard_normal()
                lines.append(f"{rng.standard_normal():.17e} {im:.17e}")
            elif field == "integer":
                lines.append(str(int(rng.integers(-9, 10))))
            else:
                lines.append(f"{rng.standard_normal():.17e}")
    path = _write(tmp_path / "b.mtx", f"%%MatrixMarket matrix array {field} {symm}", f"{n} {m}", lines)
    r = pkg.mm_read(path)
    assert r.rep == "array" and r.vals.shape == (n, m)
    np.testing.assert_array_equal(r.vals, _scipy_dense(path, field == "complex"))


def test_fortran_d_exponents_and_spread_values(pkg, tmp_path):
    path = _write(tmp_path / "d.mtx", "%%MatrixMarket matrix coordinate real general", "2 2 2",
                  ["1 1 1.5D+00", "2 2", "-2.0d-01"])
    r = pkg.mm_read(path, "crs")
    np.testing.assert_array_equal(r.vals, [1.5, -0.2])
    np.testing.assert_array_equal(r.row_ptr, [1, 2, 3])


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n",     # row out of range
    "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n",     # truncated
    "%%MatrixMarket vector coordinate real general\n2 2 1\n1 1 1.0\n",     # not a matrix
    "%%MatrixMarket matrix coordinate real hermitian\n2 2 1\n1 1 1.0\n",   # hermitian real
    "MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.0\n",       # no banner
])
def test_malformed_files_are_rejected(pkg, tmp_path, text):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    with pytest.raises(pkg.IDRSError):
        pkg.mm_read(str(p))
    with pytest.raises(pkg.IDRSError):
        pkg.mm_read(str(tmp_path / "missing.mtx"))


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="reference data not present")
@pytest.mark.parametrize("name", ["WEDGE_DATA/wedge1_K.mtx", "WEDGE_DATA/wedge2_C.mtx",
                                  "WEDGE_DATA/wedge2_M.mtx", "WEDGE_DATA/wedge1_b.mtx",
                                  "OCEAN_DATA/STOMMEL/stommel6.mtx",
                                  "OCEAN_DATA/STOMMEL/stommel6_b.mtx"])
def test_reference_example_files(pkg, name):
    """The reference's own Matrix Market examples read like scipy reads them."""
    path = os.path.join(REF_DATA, name)
    for fmt in (None, "crs"):
        r = pkg.mm_read(path, fmt)
        np.testing.assert_array_equal(_dense_from(r, r.field == "complex"),
                                      _scipy_dense(path, r.field == "complex"))


def _spread(tokens, rng):
    """tokens joined by irregular whitespace: spaces, tabs, CRLF and LF line
    breaks anywhere (list-directed input allows values spread over lines)"""
    seps = np.array([" ", "  ", "\t", "\n", "\r\n", " \n "])
    pick = rng.integers(0, len(seps), size=len(tokens))
    return "".join(t + seps[k] for t, k in zip(tokens, pick))


def test_large_coordinate_file_parsed_in_parallel(pkg, tmp_path):
    """A multi-megabyte file takes the multi-threaded scan (chunks cut at
    whitespace, tokens numbered by a prefix sum): every index and value comes
    back exactly as written, in file order."""
    rng = np.random.default_rng(11)
    n, k = 5000, 150000
    i = rng.integers(1, n + 1, size=k)
    j = rng.integers(1, n + 1, size=k)
    v = rng.standard_normal(k) * 10.0 ** rng.integers(-5, 6, size=k)
    toks = []
    for a, b, x in zip(i.tolist(), j.tolist(), v.tolist()):
        toks += [str(a), str(b), repr(x) if rng.random() < 0.9 else repr(x).replace("e", "D")]
    p = tmp_path / "big.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n% big\n" + f"{n} {n} {k}\n" + _spread(toks, rng))
    assert p.stat().st_size > 3 << 20
    r = pkg.mm_read(str(p), "coo")
    np.testing.assert_array_equal(r.indx, i)
    np.testing.assert_array_equal(r.jndx, j)
    np.testing.assert_array_equal(r.vals, v)


def test_large_complex_array_file_parsed_in_parallel(pkg, tmp_path):
    rng = np.random.default_rng(12)
    n, m = 40000, 3
    Z = rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m))
    toks = []
    for z in Z.T.ravel().tolist():
        toks += [repr(z.real), "+" + repr(z.imag) if z.imag >= 0 else repr(z.imag)]
    p = tmp_path / "bigz.mtx"
    p.write_text("%%MatrixMarket matrix array complex general\n" + f"{n} {m}\n" + _spread(toks, rng))
    assert p.stat().st_size > 2 << 20
    r = pkg.mm_read(str(p))
    np.testing.assert_array_equal(r.vals, Z.astype(np.complex64).astype(np.complex128))


@pytest.mark.parametrize("damage", ["bad_value", "bad_index", "truncated"])
def test_large_file_errors_are_reported(pkg, tmp_path, damage):
    rng = np.random.default_rng(13)
    n, k = 3000, 120000
    lines = [f"{a} {b} {x!r}" for a, b, x in zip(rng.integers(1, n + 1, size=k).tolist(),
                                                   rng.integers(1, n + 1, size=k).tolist(),
                                                   rng.standard_normal(k).tolist())]
    if damage == "bad_value":
        lines[k * 2 // 3] = "7 7 abc"  # no number (a numeric prefix is read, as strtod does)
    elif damage == "bad_index":
        lines[k // 2] = f"{n + 1} 1 1.0"
    else:
        lines = lines[:-5]
    p = tmp_path / "dmg.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n" + f"{n} {n} {k}\n" + "\n".join(lines) + "\n")
    assert p.stat().st_size > 1 << 20
    with pytest.raises(pkg.IDRSError):
        pkg.mm_read(str(p))
