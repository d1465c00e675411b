"""Sorted Coulomb matrix on the GPU: bit-exact against the oracle."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from qml_gb300 import core
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu


def run(cuda, z, r, off, size, sorting="row-norm"):
    return core.coulomb_matrix_batch(torch.from_numpy(z).to(cuda), torch.from_numpy(r).to(cuda),
                                     torch.from_numpy(off).to(cuda), size, sorting).cpu().numpy()


def test_golden_fixture(cuda, oracle):
    g = load_golden("cm_qm7_0101_0110.npz")
    size = int(g["size"])
    X = run(cuda, g["charges"], g["coordinates"], g["offsets"], size)
    U = run(cuda, g["charges"], g["coordinates"], g["offsets"], size, "unsorted")
    assert np.allclose(X, g["sorted"]) and np.allclose(U, g["unsorted"])
    Xo = oracle.cm_sorted_batch(g["charges"], g["coordinates"], g["offsets"], size)
    assert np.array_equal(X, Xo)
    off = g["offsets"]
    for m in range(len(off) - 1):
        u = oracle.cm_unsorted(g["charges"][off[m]:off[m + 1]], g["coordinates"][off[m]:off[m + 1]], size)
        assert np.array_equal(U[m], u)


@pytest.mark.parametrize("n_mol,seed", [(1, 1), (257, 2), (5000, 3)])
def test_synthetic_bit_exact(cuda, oracle, n_mol, seed):
    b = generate_molecules(n_mol, seed=seed)
    X = run(cuda, b.charges, b.coordinates, b.offsets, 23)
    assert np.array_equal(X, oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23))


def test_sizes_and_padding(cuda, oracle):
    b = generate_molecules(64, seed=9, max_atoms=23)
    for size in (23, 24, 32):
        X = run(cuda, b.charges, b.coordinates, b.offsets, size)
        assert np.array_equal(X, oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, size))
    b = generate_molecules(40, seed=4, min_atoms=32, max_atoms=32)
    X = run(cuda, b.charges, b.coordinates, b.offsets, 32)
    assert np.array_equal(X, oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 32))


def test_ties_and_single_atoms(cuda, oracle):
    z = np.array([1.0, 6.0, 1.0, 8.0, 1.0, 1.0, 1.0])
    r = np.array([[-1.1, 0, 0], [0, 0, 0], [1.1, 0, 0], [5, 5, 5], [0, 0, 0], [9, 9, 9], [9, 9, 10.5]])
    off = np.array([0, 3, 4, 5, 7], dtype=np.int64)
    X = run(cuda, z, r, off, 4)
    assert np.array_equal(X, oracle.cm_sorted_batch(z, r, off, 4))


def test_empty_batch_and_errors(cuda):
    out = run(cuda, np.zeros(0), np.zeros((0, 3)), np.zeros(1, dtype=np.int64), 23)
    assert out.shape == (0, 276)
    b = generate_molecules(3, seed=1, min_atoms=10, max_atoms=10)
    with pytest.raises(RuntimeError):
        run(cuda, b.charges, b.coordinates, b.offsets, 9)


def test_dropin_single_molecule_and_compound(cuda, oracle, tmp_path):
    from qml_gb300.compound import Compound
    from qml_gb300.representations import generate_coulomb_matrix
    b = generate_molecules(5, seed=21)
    for m in range(5):
        z, r = b.molecule(m)
        assert np.array_equal(generate_coulomb_matrix(z.astype(int), r, size=23),
                              oracle.cm_sorted(z, r, 23))
    p = tmp_path / "m.xyz"
    p.write_text("3\n\nO 0.0 0.0 0.1\nH 0.75 0.0 -0.4\nH -0.75 0.0 -0.4\n")
    c = Compound(xyz=str(p))
    c.generate_coulomb_matrix(size=5, sorting="row-norm")
    assert np.array_equal(c.representation, oracle.cm_sorted(c.nuclear_charges, c.coordinates, 5))
