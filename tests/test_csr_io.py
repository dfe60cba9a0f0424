"""CSR matrix files (GCGE_CUDA_CSR_ReadFile / WriteText / WriteBinary) on the
host, no GPU: the reference's own data files read in both formats agree
bit-exact with each other and with independent numpy parses; written files
read back bit-exact; malformed files fail with GCGE_CUDA_ERR_IO and a reason."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

DATA = os.path.join(GOLDEN, "csr_files")


@pytest.fixture(scope="module")
def io():
    from gcge_old_gb300 import lib as L
    L.load(build_if_missing=True)
    from gcge_old_gb300 import csr_io
    return csr_io


def petsc_numpy(path):
    """PETSc binary Mat parsed with numpy (big-endian int32 header, row lengths
    and columns, big-endian float64 values)."""
    b = open(path, "rb").read()
    cid, m, n, nz = np.frombuffer(b[:16], ">i4")
    assert cid == 1211216
    rl = np.frombuffer(b[16:16 + 4 * m], ">i4")
    o = 16 + 4 * m
    col = np.frombuffer(b[o:o + 4 * nz], ">i4")
    val = np.frombuffer(b[o + 4 * nz:o + 12 * nz], ">f8")
    return np.concatenate([[0], np.cumsum(rl)]), col, val


def same(A, rp, col, val):
    np.testing.assert_array_equal(A.rowptr, rp)
    np.testing.assert_array_equal(A.col, col)
    assert A.val.tobytes() == np.asarray(val, dtype=np.float64).tobytes()


def test_reference_files_text_and_binary_agree(io):
    from gcge_old_gb300.matrices import read_csr_text
    At = io.read_csr(os.path.join(DATA, "A_5.txt"))
    Ab = io.read_csr(os.path.join(DATA, "A_5.petsc.bin"))
    assert At.n == 1089 and At.nnz == 7361
    same(Ab, *petsc_numpy(os.path.join(DATA, "A_5.petsc.bin")))
    same(At, Ab.rowptr, Ab.col, Ab.val)
    for f in ("A_3.txt", "A_5.txt"):
        P = read_csr_text(os.path.join(DATA, f))
        same(io.read_csr(os.path.join(DATA, f)), P.rowptr, P.col, P.val)


def test_round_trips_are_bit_exact(io, tmp_path):
    from gcge_old_gb300.matrices import diffusion27
    A, B = diffusion27(m=12, seed=2)
    rng = np.random.default_rng(0)
    A.val[:50] = rng.standard_normal(50) * 10.0 ** rng.integers(-300, 300, 50)  # extreme exponents
    for w in (io.write_csr_text, io.write_csr_binary):
        p = tmp_path / ("m" + w.__name__)
        w(p, A)
        same(io.read_csr(p), A.rowptr, A.col, A.val)
    io.write_csr_binary(tmp_path / "b.bin", A)
    same(io.read_csr(tmp_path / "b.bin"), *petsc_numpy(tmp_path / "b.bin"))


def test_empty_and_ragged(io, tmp_path):
    from gcge_old_gb300.matrices import CSRMatrix
    p = tmp_path / "z.txt"
    p.write_text("0 0 0\n0\n")
    Z = io.read_csr(p)
    assert Z.n == 0 and Z.nnz == 0
    # empty rows, tabs and CRLF line ends, extra trailing tokens (ignored)
    p.write_text("3\r\n3\r\n2\r\n0\t0 1 2\n2\n0\n-1.5e-3 2.25\n99 junk\n")
    A = io.read_csr(p)
    same(A, [0, 0, 1, 2], [2, 0], [-1.5e-3, 2.25])
    E = CSRMatrix(4, np.array([0, 0, 0, 1, 1], np.int32), np.array([3], np.int32),
                  np.array([7.0]))
    io.write_csr_binary(tmp_path / "e.bin", E)
    same(io.read_csr(tmp_path / "e.bin"), E.rowptr, E.col, E.val)


def test_large_text_parses_in_parallel_ranges(io, tmp_path):
    """Several MiB of text: the byte ranges of the parallel parser cut tokens only
    at whitespace."""
    import scipy.sparse as sp
    from gcge_old_gb300.matrices import CSRMatrix
    rng = np.random.default_rng(1)
    M = sp.random(20000, 20000, density=2e-3, random_state=3, format="csr")
    M.data = rng.standard_normal(M.nnz) * 1e5
    A = CSRMatrix.from_scipy(M)
    io.write_csr_text(tmp_path / "big.txt", A)
    assert os.path.getsize(tmp_path / "big.txt") > 8 << 20
    same(io.read_csr(tmp_path / "big.txt"), A.rowptr, A.col, A.val)


@pytest.mark.parametrize("text,why", [
    ("", "bad header"),
    ("2 2\n", "bad header"),
    ("2 2 2\n0 1 2\n0 1\n1.0\n", "file ends"),
    ("2 2 2\n0 1 2\n0 1\n1.0 x\n", "malformed number in val"),
    ("2 2 2\n0 1 2\n0 1.5\n1 2\n", "malformed number in col"),
    ("2 2 2\n1 1 2\n0 1\n1 2\n", "start at 0"),
    ("2 2 2\n0 2 1\n0 1\n1 2\n", "decrease"),
    ("2 2 2\n0 1 1\n0 1\n1 2\n", "differs from nnz"),
    ("2 2 2\n0 1 2\n0 2\n1 2\n", "out of range"),
    ("2 2 2\n0 1 2\n0 1\n1 1e999\n", "malformed number in val"),
])
def test_malformed_text_is_rejected(io, tmp_path, text, why):
    from gcge_old_gb300 import lib as L
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(L.GcgeCudaError, match=why) as e:
        io.read_csr(p)
    assert "file error (6)" in str(e.value)


def test_malformed_binary_is_rejected(io, tmp_path):
    from gcge_old_gb300 import lib as L
    good = open(os.path.join(DATA, "A_5.petsc.bin"), "rb").read()
    cases = [(good[:12], "header truncated"), (good[:-8], "ends before"),
             (good[:16] + b"\x7f\xff\xff\xff" + good[20:], "row lengths")]
    for blob, why in cases:
        p = tmp_path / "bad.bin"
        p.write_bytes(blob)
        with pytest.raises(L.GcgeCudaError, match=why):
            io.read_csr(p)
    with pytest.raises(L.GcgeCudaError, match="cannot open"):
        io.read_csr(tmp_path / "missing.txt")


def test_reference_reader_agrees(io, tmp_path):
    """The reference's own CSR_ReadMatFile (built from its sources into
    oracle/_ref) reads what the native text writer wrote, and reads the
    reference's data file, to the same bits as the native reader."""
    from oracle import oracle as O
    if not O.ref_available():
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    from gcge_old_gb300.matrices import diffusion27
    A, _ = diffusion27(m=10, seed=4)
    io.write_csr_text(tmp_path / "w.txt", A)
    for p in (tmp_path / "w.txt", os.path.join(DATA, "A_5.txt")):
        n, nc, rp, col, val = O.ref_read_csr(str(p))
        M = io.read_csr(p)
        assert n == nc == M.n
        same(M, rp, col, val)
