"""Matrix Market I/O (src/generators/mtx_io.cu): the library's reader and
writer against a numpy restatement of the reference's reader, exact round
trips, error cases, and (with the reference sources present) the reference's
own readMTXFile on the same files."""
from __future__ import annotations

import numpy as np
import pytest

import muxi_spmv_gb300 as mx


def restate(text: str, expand: bool = True):
    """numpy restatement of readMTXFile (mtx_io.cu:111-222): 1-based entries,
    pattern -> 1, symmetric mirrored, stable sort by (row, column)."""
    lines = text.splitlines()
    banner = lines[0].lower().split()
    sym = "symmetric" in banner
    pattern = "pattern" in banner
    body = [l for l in lines[1:] if l.strip() and not l.lstrip().startswith("%")]
    R, Cc, n = (int(t) for t in body[0].split())
    rows, cols, vals = [], [], []
    for l in body[1:1 + n]:
        t = l.split()
        r, c = int(t[0]) - 1, int(t[1]) - 1
        v = 1.0 if pattern else float(t[2])
        rows.append(r), cols.append(c), vals.append(v)
        if sym and expand and r != c:
            rows.append(c), cols.append(r), vals.append(v)
    rows, cols, vals = np.array(rows, np.int64), np.array(cols, np.int64), np.array(vals)
    order = np.lexsort((np.arange(len(rows)), cols, rows))  # stable by (row, col)
    rp = np.zeros(R + 1, np.int32)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols[order].astype(np.int32), vals[order], Cc


FILES = {
    "general": "%%MatrixMarket matrix coordinate real general\n% a comment\n4 5 6\n1 1 1.5\n3 2 -2\n1 5 3.25\n"
               "2 3 4e-3\n4 4 7\n3 1 0.5\n",
    "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n3 3 4\n1 1 2\n2 1 -1\n3 2 -1\n3 3 2\n",
    "pattern": "%%MatrixMarket matrix coordinate pattern general\n%\n%\n3 4 3\n2 4\n1 1\n3 2\n",
    "integer_sym": "%%MatrixMarket matrix coordinate integer symmetric\n4 4 3\n4 1 5\n2 2 -3\n3 2 9\n",
    "blank_lines": "%%MatrixMarket matrix coordinate real general\n\n2 2 2\n\n2 2 1.0\n% mid comment\n1 2 2.0\n",
    "empty_rows": "%%MatrixMarket matrix coordinate real general\n6 3 2\n5 3 1\n2 1 2\n",
}


@pytest.mark.parametrize("name", sorted(FILES))
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_reader_matches_restatement(tmp_path, name, dtype):
    f = tmp_path / f"{name}.mtx"
    f.write_text(FILES[name])
    for expand in (True, False):
        A = mx.readMTXFile(f, dtype, expandSymmetric=expand)
        rp, ci, v, cols = restate(FILES[name], expand)
        assert A.numCols == cols
        np.testing.assert_array_equal(A.rowPtr, rp)
        np.testing.assert_array_equal(A.colIdx, ci)
        np.testing.assert_array_equal(A.values, v.astype(dtype))
    h = mx.readMTXHeader(f)
    assert h["numCols"] == cols and h["nnz"] == int([l for l in FILES[name].splitlines()[1:]
                                                      if l.strip() and not l.startswith("%")][0].split()[2])


def test_duplicates_keep_file_order(tmp_path):
    f = tmp_path / "dup.mtx"
    f.write_text("%%MatrixMarket matrix coordinate real general\n2 2 4\n1 2 3\n1 2 1\n2 1 5\n1 2 2\n")
    A = mx.readMTXFile(f, np.float64)
    np.testing.assert_array_equal(A.rowPtr, [0, 3, 4])
    np.testing.assert_array_equal(A.colIdx, [1, 1, 1, 0])
    np.testing.assert_array_equal(A.values, [3, 1, 2, 5])


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_round_trip_is_exact(tmp_path, dtype):
    from muxi_spmv_gb300 import workloads as W
    s = W.scaled("powerlaw8m", 3000, seed=11)
    rp, ci, v = mx.generate(s, dtype=dtype)
    A = mx.CSRMatrix(rp, ci, v, s.numCols)
    f = tmp_path / "rt.mtx"
    mx.writeMTXFile(f, A)
    assert f.read_text().startswith("%%MatrixMarket matrix coordinate real general\n")
    B = mx.readMTXFile(f, dtype)
    np.testing.assert_array_equal(B.rowPtr, rp)
    np.testing.assert_array_equal(B.colIdx, ci)
    np.testing.assert_array_equal(B.values, v)


def test_symmetric_write_then_expand(tmp_path):
    f = tmp_path / "s.mtx"
    f.write_text(FILES["symmetric"])
    A = mx.readMTXFile(f, np.float64)
    g = tmp_path / "s2.mtx"
    mx.writeMTXFile(g, A, writeSymmetric=True)  # upper triangle, as the reference writes it
    B = mx.readMTXFile(g, np.float64)
    np.testing.assert_array_equal(B.rowPtr, A.rowPtr)
    np.testing.assert_array_equal(B.colIdx, A.colIdx)
    np.testing.assert_array_equal(B.values, A.values)


@pytest.mark.parametrize("text,status", [
    ("%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n", -8),
    ("%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n", -2),       # the reference writer's banner
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", -2),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n", -2),     # row outside the shape
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1\n", -2),     # truncated
    ("%%MatrixMarket matrix coordinate real general\nx y z\n", -2),
])
def test_reader_refuses(tmp_path, text, status):
    f = tmp_path / "bad.mtx"
    f.write_text(text)
    with pytest.raises(mx.SpmvError) as e:
        mx.readMTXFile(f)
    assert e.value.status == status
    with pytest.raises(mx.SpmvError):
        mx.readMTXFile(tmp_path / "missing.mtx")


@pytest.mark.refsrc
@pytest.mark.parametrize("name", ["general", "symmetric", "pattern", "integer_sym", "empty_rows"])
def test_reader_matches_reference_reader(tmp_path, name):
    refpin = pytest.importorskip("oracle.refpin")
    if not refpin.available():
        pytest.skip("reference sources not present")
    f = tmp_path / f"{name}.mtx"
    f.write_text(FILES[name])
    st, rp, ci, v, cols = refpin.mtx_read(f)
    assert st == 0
    A = mx.readMTXFile(f, np.float64)
    assert A.numCols == cols
    np.testing.assert_array_equal(A.rowPtr, rp)
    np.testing.assert_array_equal(A.colIdx, ci)
    np.testing.assert_array_equal(A.values, v)


@pytest.mark.refsrc
def test_reference_reader_on_a_large_written_file(tmp_path):
    """A 20,000-row power-law matrix written by this library, read by both."""
    refpin = pytest.importorskip("oracle.refpin")
    if not refpin.available():
        pytest.skip("reference sources not present")
    from muxi_spmv_gb300 import workloads as W
    s = W.scaled("powerlaw8m", 20000, seed=5)
    rp, ci, v = mx.generate(s, dtype=np.float64)
    f = tmp_path / "big.mtx"
    mx.writeMTXFile(f, mx.CSRMatrix(rp, ci, v, s.numCols))
    st, rrp, rci, rv, cols = refpin.mtx_read(f)
    assert st == 0
    np.testing.assert_array_equal(rrp, rp)
    np.testing.assert_array_equal(rci, ci)
    # The law repeats some (row, column) pairs; the reference's std::sort leaves
    # their order unspecified, so each repeated group is compared as a multiset.
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    a = np.lexsort((v, ci, rows))
    b = np.lexsort((rv, rci, rows))
    np.testing.assert_array_equal(rv[b], v[a])
    B = mx.readMTXFile(f, np.float64)  # this library keeps file order for repeats
    np.testing.assert_array_equal(B.values, v)
