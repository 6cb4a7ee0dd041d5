"""Input files on the host: the Matrix Market reader, the CSV right-hand-side
reader and the row-block split, against the reference's own readers
(src/readMTX.c:8-135 + src/matrixType.c:4-52, src/common.c:16-48) through the
committed fixtures (tests/golden/make_io_golden.py) and, where the reference
sources are present, live; the splits against a restatement of
src/SparseMatrixDistribution.c:64-124 and src/GetRHS.c:139-202."""
import os

import numpy as np
import pytest

import cacg_gb300 as cg
import oracle as O
from cacg_gb300 import _lib as L

HERE = os.path.dirname(os.path.abspath(__file__))
IO = os.path.join(HERE, "golden", "io")
GOLD = np.load(os.path.join(HERE, "golden", "io_golden.npz"))
MTX = sorted(f[:-4] for f in os.listdir(IO) if f.endswith(".mtx"))


@pytest.mark.parametrize("name", MTX)
def test_read_mtx_matches_reference_fixture(name):
    rp, ci, v, shape = cg.read_mtx(os.path.join(IO, name + ".mtx"))
    assert np.array_equal(rp, GOLD[name + "/rp"])
    assert np.array_equal(ci, GOLD[name + "/ci"])
    assert np.array_equal(v, GOLD[name + "/v"])
    assert tuple(shape) == tuple(GOLD[name + "/shape"])


@pytest.mark.skipif(not O.ref_available(), reason="reference sources absent")
def test_read_mtx_matches_reference_live(tmp_path):
    # a symmetric stencil written in random entry order, read by both
    rp, ci, v = cg.gen_matrix("lap3d7", 9, shift=0.25)
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    low = rows >= ci
    order = np.random.default_rng(3).permutation(int(low.sum()))
    I, J, V = rows[low][order], ci[low][order], v[low][order]
    p = tmp_path / "a.mtx"
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n")
        f.write("%d %d %d\n" % (n, n, len(I)))
        for i, j, x in zip(I, J, V):
            f.write("%d %d %.17g\n" % (i + 1, j + 1, x))
    ours = cg.read_mtx(str(p))
    ref = O.ref_read_mtx(str(p))
    for a, b in zip(ours[:3], ref[:3]):
        assert np.array_equal(a, b)
    assert ours[3] == ref[3]
    # same matrix as the generator's (row order may differ within a row)
    for r in range(n):
        a = sorted(zip(ours[1][ours[0][r]:ours[0][r + 1]], ours[2][ours[0][r]:ours[0][r + 1]]))
        b = sorted(zip(ci[rp[r]:rp[r + 1]], v[rp[r]:rp[r + 1]]))
        assert a == b


@pytest.mark.parametrize("text,code", [
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1\n", L.ERR_ARG),   # short entry
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", L.ERR_ARG),  # row > M
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", L.ERR_ARG),  # truncated
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", L.ERR_UNSUPPORTED),
    ("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n", L.ERR_UNSUPPORTED),
    ("%%MatrixMarket matrix coordinate real hermitian\n1 1 1\n1 1 1\n", L.ERR_ARG),
    ("%%MatrixMarket matrix coordinate pattern skew-symmetric\n1 1 0\n", L.ERR_ARG),
    ("%%NotMatrixMarket matrix coordinate real general\n1 1 0\n", L.ERR_ARG),
    ("%%MatrixMarket matrix coordinate real general\n% no size line\n", L.ERR_ARG),
])
def test_read_mtx_errors(tmp_path, text, code):
    p = tmp_path / "bad.mtx"
    p.write_text(text)
    with pytest.raises(cg.CacgError) as e:
        cg.read_mtx(str(p))
    assert e.value.code == code
    with pytest.raises(cg.CacgError):
        cg.read_mtx(str(tmp_path / "missing.mtx"))


def test_read_mtx_empty_and_blank_lines(tmp_path):
    p = tmp_path / "e.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n%\n\n3 4 0\n")
    rp, ci, v, shape = cg.read_mtx(str(p))
    assert shape == (3, 4) and rp.tolist() == [0, 0, 0, 0] and len(ci) == 0


def _row_block_restated(n, myid, numprocs):
    """src/SparseMatrixDistribution.c:72-78 / src/GetRHS.c:147-150"""
    per = n // numprocs
    cnt = n - per * (numprocs - 1) if myid == numprocs - 1 else per
    return myid * per, cnt


@pytest.mark.parametrize("numprocs", [1, 2, 3, 5, 8])
def test_csr_row_block(numprocs):
    rp, ci, v, (nr, nc) = cg.read_mtx(os.path.join(IO, "lap2d_12_sym.mtx"))
    rows_seen = 0
    for myid in range(numprocs):
        lrp, lci, lv, start = cg.csr_row_block(rp, ci, v, nc, myid, numprocs)
        r0, cnt = _row_block_restated(nr, myid, numprocs)
        assert start == r0 and len(lrp) == cnt + 1 and lrp[0] == 0
        assert np.array_equal(lrp, rp[r0:r0 + cnt + 1] - rp[r0])
        assert np.array_equal(lci, ci[rp[r0]:rp[r0 + cnt]])
        assert np.array_equal(lv, v[rp[r0]:rp[r0 + cnt]])
        rows_seen += cnt
    assert rows_seen == nr
    with pytest.raises(cg.CacgError):
        cg.csr_row_block(rp, ci, v, nc, 3, 3)


def test_read_csv_matches_reference_fixture():
    B, got = cg.read_csv(os.path.join(IO, "rhs_144x4.csv"), 144, 4)
    assert got == 144 and np.array_equal(B, GOLD["rhs_144x4"])
    S, got = cg.read_csv(os.path.join(IO, "rhs_short.csv"), 8, 3)
    assert got == 5 and np.array_equal(S, GOLD["rhs_short"]) and not S[5:].any()


@pytest.mark.skipif(not O.ref_available(), reason="reference sources absent")
def test_read_csv_matches_reference_live(tmp_path):
    X = np.random.default_rng(11).normal(size=(50, 16)) * 10.0 ** np.arange(-8, 8)
    p = tmp_path / "r.csv"
    with open(p, "w") as f:
        for row in X:
            f.write(",".join("%.18e" % x for x in row) + "\n")
    ours, got = cg.read_csv(str(p), 50, 16)
    assert got == 50
    assert np.array_equal(ours, O.ref_parse_csv(str(p), 50, 16))
    assert np.array_equal(ours, X)  # %.18e round-trips FP64


def test_read_csv_errors(tmp_path):
    p = tmp_path / "bad.csv"
    p.write_text("1,2,3\n4,5\n")
    with pytest.raises(cg.CacgError) as e:
        cg.read_csv(str(p), 2, 3)
    assert e.value.code == L.ERR_ARG
    with pytest.raises(cg.CacgError):
        cg.read_csv(str(tmp_path / "missing.csv"), 1, 1)
    # lines longer than the reference's 1024-byte buffer are read whole
    q = tmp_path / "wide.csv"
    row = np.arange(200, dtype=np.float64) / 7.0
    q.write_text(",".join("%.18e" % x for x in row) + "\n")
    A, got = cg.read_csv(str(q), 1, 200)
    assert got == 1 and np.array_equal(A[0], row)


@pytest.mark.parametrize("numprocs", [1, 2, 4, 7])
def test_dense_row_block(numprocs):
    B = GOLD["rhs_144x4"]
    for myid in range(numprocs):
        blk, f = cg.dense_row_block(B, myid, numprocs)
        r0, cnt = _row_block_restated(144, myid, numprocs)
        assert np.array_equal(blk, B[r0:r0 + cnt])
        assert f == {"local_num_row": cnt, "local_num_col": 4, "global_num_row": 144,
                     "global_num_col": 4, "start_idx": myid * 4 * (144 // numprocs)}
