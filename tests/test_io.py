"""Batched XYZ ingestion and KRR model files (host side; no GPU)."""
import numpy as np
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
