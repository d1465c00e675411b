"""Batched XYZ ingestion and KRR model files (host side; no GPU)."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from qml_gb300.compound import Compound
from qml_gb300.io import load_krr, read_xyz_batch, save_krr
from qml_gb300.krr import KRR

SYMBOL = {1: "H", 6: "C", 7: "N", 8: "O", 16: "S"}


def write_fixture_xyz(tmp_path):
    g = load_golden("cm_qm7_0101_0110.npz")
    z, r, off = g["charges"], g["coordinates"], g["offsets"]
    paths = []
    for m in range(len(off) - 1):
        p = tmp_path / ("%04d.xyz" % (101 + m))
        lines = ["%d" % (off[m + 1] - off[m]), "comment"]
        for a in range(off[m], off[m + 1]):
            lines.append("%s %.17g %.17g %.17g" % (SYMBOL[int(z[a])], *r[a]))
        p.write_text("\n".join(lines) + "\n")
        paths.append(str(p))
    return paths, z, r, off


def test_read_xyz_batch_round_trip(tmp_path):
    paths, z, r, off = write_fixture_xyz(tmp_path)
    b = read_xyz_batch(paths)
    assert np.array_equal(b.offsets, off)
    assert np.array_equal(b.charges, z) and np.array_equal(b.coordinates, r)
    # the same as one Compound per file
    for m, p in enumerate(paths):
        c = Compound(xyz=p)
        assert np.array_equal(c.nuclear_charges, z[off[m]:off[m + 1]])
        assert np.array_equal(c.coordinates, r[off[m]:off[m + 1]])
    # the parallel path keeps the input order
    many = paths * 20
    bm = read_xyz_batch(many, workers=4)
    assert bm.n_mol == len(many) and np.array_equal(bm.charges, np.tile(z, 20))


def test_krr_file_round_trip(tmp_path):
    m = KRR(kernel="laplacian", sigma=123.0, lam=1e-6, precision="fp64")
    m.X = torch.arange(12, dtype=torch.float64).reshape(4, 3)
    m.alpha = torch.tensor([1.0, -2.0, 3.5, 0.25], dtype=torch.float64)
    path = str(tmp_path / "model.npz")
    save_krr(path, m)
    r = load_krr(path, device="cpu")
    assert (r.kernel, r.sigma, r.lam, r.precision) == ("laplacian", 123.0, 1e-6, "fp64")
    assert torch.equal(r.X, m.X) and torch.equal(r.alpha, m.alpha)


# (text, what read_xyz gives or raises): each case goes through the native reader
# and parser, alone and inside a larger batch, and must agree with read_xyz
EDGE_CASES = [
    "3\ncomment\nO 0.0 0.0 0.1\nH 0.7 0.0 -0.5\nH -0.7 0.0 -0.5\n",
    "2\r\nCRLF line ends\r\nC 1 2 3\r\nN 4 5 6\r\n",
    "2\rlone CR\rC 1 2 3\rN 4 5 6",
    "  +2 \n\nC\t1.5\t-2.25e-3\t3E2 extra fields\n\x0bN 4 5 6\x0c\n",
    "5\nmore atoms counted than lines\nC 1 2 3\nH 1 1 1\n",
    "4\nstops at a short line\nC 1 2 3\nH 1 1\nO 7 7 7\n",
    "0\nno atoms\n",
    "1",
    "3\nno trailing newline\nUuq 1 2 3\nCn 4 5 6\nUuh 7 8 9",
    "2\nnan and inf\nC nan -inf 1\nH Infinity +0.5 -0\n",
    "1\ncomment with é (UTF-8)\nC 1 2 3\n",
    "1\nunderscores float() reads\nC 1_000.5 2 3\n",
    "2\nPython int() reads 014\nC 1 2 3\nH 4 5 6\n".replace("2\n", "014\n", 1),
]
BAD_CASES = [
    ("1\nunknown element\nXx 1 2 3\n", KeyError),
    ("1\nhex is not a float\nC 0x10 2 3\n", ValueError),
    ("1\nnan(...) is not a float\nC nan(1) 2 3\n", ValueError),
    ("-1\nnegative count\nC 1 2 3\n", ValueError),
    ("two\nnot a count\nC 1 2 3\n", ValueError),
    ("", IndexError),
]


def _same(a, b):
    return np.array_equal(a.view(np.int64), b.view(np.int64))


def test_read_xyz_batch_edge_cases(tmp_path):
    from qml_gb300.io import read_xyz
    paths = []
    for i, text in enumerate(EDGE_CASES):
        p = tmp_path / ("edge%02d.xyz" % i)
        p.write_bytes(text.encode("utf-8"))
        paths.append(str(p))
    want = [read_xyz(p) for p in paths]
    for workers in (1, 0):
        for batch in (paths, paths * 40):
            b = read_xyz_batch(batch, workers=workers)
            assert b.n_mol == len(batch)
            for m in range(b.n_mol):
                z, r = b.molecule(m)
                wz, wr = want[m % len(paths)]
                assert _same(z, wz) and _same(r, wr.reshape(-1, 3)), (m, batch[m])
    assert read_xyz_batch([]).n_mol == 0


def test_read_xyz_batch_errors_are_the_reference_ones(tmp_path):
    good = tmp_path / "good.xyz"
    good.write_text(EDGE_CASES[0])
    for i, (text, exc) in enumerate(BAD_CASES):
        p = tmp_path / ("bad%02d.xyz" % i)
        p.write_text(text)
        with pytest.raises(exc):
            read_xyz_batch([str(good)] * 100 + [str(p)])
    with pytest.raises(FileNotFoundError):
        read_xyz_batch([str(good), str(tmp_path / "missing.xyz")])
    # not a regular file: the native reader gives it no bytes, read_xyz raises
    (tmp_path / "adir.xyz").mkdir()
    with pytest.raises(IsADirectoryError):
        read_xyz_batch([str(good), str(tmp_path / "adir.xyz")])


def test_native_parser_flags_instead_of_guessing():
    # the C entry point alone: flagged files get an empty range, the others parse
    from qml_gb300 import _lib
    lib = _lib.load()
    files = [b"1\n\nC 1 2 3\n", b"1\n\nC 1_0 2 3\n", b"2\n\nH 1 2 3\nO 4 5 6\n",
             b"1\n\xc3\xa9\nC 1 2 3\n"]
    text = np.frombuffer(b"".join(files), dtype=np.uint8).copy()
    starts = np.zeros(len(files) + 1, dtype=np.int64)
    starts[1:] = np.cumsum([len(f) for f in files])
    cap = 16
    z = np.zeros(cap)
    r = np.zeros((cap, 3))
    off = np.zeros(len(files) + 1, dtype=np.int64)
    st = np.zeros(len(files), dtype=np.int32)
    assert lib.qmlg_parse_xyz(text.ctypes.data, starts.ctypes.data, len(files), 2,
                              off.ctypes.data, st.ctypes.data, z.ctypes.data, r.ctypes.data,
                              cap) == 0
    # file 1 passes the count phase (its number fails only when parsed), so it keeps
    # its one-atom range; file 3 (non-ASCII) is flagged before it gets a range
    assert st.tolist() == [0, 1, 0, 1]
    assert off.tolist() == [0, 1, 2, 4, 4]
    assert z[[0, 2, 3]].tolist() == [6.0, 1.0, 8.0]
    assert r[3].tolist() == [4.0, 5.0, 6.0]
    # too little room, and bad arguments
    assert lib.qmlg_parse_xyz(text.ctypes.data, starts.ctypes.data, len(files), 1,
                              off.ctypes.data, st.ctypes.data, z.ctypes.data, r.ctypes.data,
                              2) == -7
    assert lib.qmlg_parse_xyz(None, starts.ctypes.data, len(files), 1, off.ctypes.data,
                              st.ctypes.data, z.ctypes.data, r.ctypes.data, cap) == -1
