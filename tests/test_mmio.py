"""MatrixMarket ingestion (race_gb300/mmio.py) with the semantics of RACE's
example driver: sparsemat::readFile (symmetric expansion, stable row sort,
pattern value 0.01) and makeDiagFirst."""
import gzip
import os
import pathlib

import numpy as np
import pytest

from race_gb300 import mmio
from race_gb300.matgen import Csr


def _write(tmp_path, name, text, gz=False):
    p = tmp_path / name
    if gz:
        with gzip.open(p, "wt") as f:
            f.write(text)
    else:
        p.write_text(text)
    return p


def test_general_real_rows_sorted_stably(tmp_path):
    p = _write(tmp_path, "g.mtx", """%%MatrixMarket matrix coordinate real general
% a comment
3 3 5
3 1 5.0
1 2 1.5
3 3 6.0
1 1 2.0
2 2 -4.0
""")
    A = mmio.read_matrix_market(p)
    assert A.n == 3
    np.testing.assert_array_equal(A.row_ptr, [0, 2, 3, 5])
    np.testing.assert_array_equal(A.col, [1, 0, 1, 0, 2])  # file order inside each row
    np.testing.assert_array_equal(A.val, [1.5, 2.0, -4.0, 5.0, 6.0])


def test_symmetric_expanded_mirror_after_entry(tmp_path):
    text = """%%MatrixMarket matrix coordinate real symmetric
3 3 4
1 1 4.0
2 1 -1.0
3 2 -2.0
3 3 4.0
"""
    for gz in (False, True):
        A = mmio.read_matrix_market(_write(tmp_path, "s.mtx.gz" if gz else "s.mtx", text, gz))
        np.testing.assert_array_equal(A.row_ptr, [0, 2, 4, 6])
        # row 0: (0,0) then the mirror (0,1) of (1,0); row 1: (1,0) then mirror (1,2); row 2: (2,1), (2,2)
        np.testing.assert_array_equal(A.col, [0, 1, 0, 2, 1, 2])
        np.testing.assert_array_equal(A.val, [4.0, -1.0, -1.0, -2.0, -2.0, 4.0])


def test_pattern_values(tmp_path):
    A = mmio.read_matrix_market(_write(tmp_path, "p.mtx", """%%MatrixMarket matrix coordinate pattern general
2 2 3
1 1
2 1
2 2
"""))
    np.testing.assert_array_equal(A.val, [0.01, 0.01, 0.01])
    np.testing.assert_array_equal(A.col, [0, 0, 1])


@pytest.mark.parametrize("header,body", [
    ("%%MatrixMarket matrix coordinate complex general", "1 1 1\n1 1 1.0 0.0\n"),
    ("%%MatrixMarket matrix coordinate integer general", "1 1 1\n1 1 3\n"),
    ("%%MatrixMarket matrix array real general", "1 1\n1.0\n"),
    ("%%MatrixMarket matrix coordinate real skew-symmetric", "2 2 1\n2 1 1.0\n"),
    ("%%MatrixMarket matrix coordinate real general", "2 3 1\n1 1 1.0\n"),
    ("%%MatrixMarket matrix coordinate real general", "2 2 3\n1 1 1.0\n"),
])
def test_rejected_files(tmp_path, header, body):
    with pytest.raises(ValueError):
        mmio.read_matrix_market(_write(tmp_path, "x.mtx", header + "\n" + body))


def test_make_diag_first():
    # row 0: diagonal in the middle; row 1: no diagonal; row 2: diagonal first
    A = Csr(3, np.array([0, 3, 4, 6], np.int32), np.array([2, 0, 1, 0, 2, 1], np.int32),
            np.array([1.0, 5.0, 2.0, 3.0, 7.0, -1.0]))
    B = mmio.make_diag_first(A, missing_diag_value=0.5)
    np.testing.assert_array_equal(B.row_ptr, [0, 3, 5, 7])
    np.testing.assert_array_equal(B.col, [0, 2, 1, 1, 0, 2, 1])
    np.testing.assert_array_equal(B.val, [5.0, 1.0, 2.0, 0.5, 3.0, 7.0, -1.0])
    C = mmio.make_diag_first(A, rewrite_all_diag_with_max_row_sum=True)
    # row sums after the insertion: 8, 3, 6 -> every diagonal becomes 8
    np.testing.assert_array_equal(C.val[C.row_ptr[:-1]], [8.0, 8.0, 8.0])
    np.testing.assert_array_equal(C.col, B.col)


def test_reference_example_matrix():
    """The reference's bundled example (examples/matrices/spinSZ12.mm.gz,
    924 rows), where this container has the reference: the same entries as
    SciPy's reader, each row in file order, and every row gets a diagonal."""
    ref = pathlib.Path(os.environ.get("RACE_REFERENCE_DIR", "/root/reference"))
    path = ref / "examples" / "matrices" / "spinSZ12.mm.gz"
    if not path.exists():
        pytest.skip("reference example matrix not present")
    scipy_io = pytest.importorskip("scipy.io")
    A = mmio.read_matrix_market(path)
    S = scipy_io.mmread(str(path)).tocsr()
    assert A.n == S.shape[0] == 924
    D = np.zeros(S.shape)
    rows = np.repeat(np.arange(A.n), np.diff(A.row_ptr))
    np.add.at(D, (rows, A.col), A.val)
    np.testing.assert_array_equal(D, S.toarray())
    B = mmio.make_diag_first(A)
    assert all(B.col[B.row_ptr[r]] == r for r in range(B.n))


def test_rcm_initial_permutation_reduces_bandwidth(mats):
    """rcm_perm gives a permutation (and its inverse) that shrinks the
    bandwidth of a scrambled banded matrix."""
    pytest.importorskip("scipy")
    A = mats["band_5k"]
    perm, inv = mmio.rcm_perm(A)
    assert np.array_equal(np.sort(perm), np.arange(A.n))
    assert np.array_equal(inv[perm], np.arange(A.n))

    def bandwidth(M):
        r = np.repeat(np.arange(M.n), np.diff(M.row_ptr))
        return int(np.max(np.abs(r - M.col)))

    assert bandwidth(A.permuted(perm, inv)) < bandwidth(A) / 10
