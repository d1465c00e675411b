"""Drop-ins for qml.wrappers.get_atomic_kernels_gaussian / _laplacian
(qml/wrappers.py:33-96): local kernels over lists of Compound objects whose
representation holds one atomic representation row per atom.  The reference pads the
rows into a (molecules, max atoms, size) array; the sums over atom pairs are the same,
so these concatenate the rows and call the local kernels.
"""
from __future__ import annotations

import numpy as np

from .kernels import get_local_kernels_gaussian, get_local_kernels_laplacian


def _stack(mols):
    n = np.array([mol.natoms for mol in mols], dtype=np.int64)
    X = np.concatenate([np.asarray(mol.representation, dtype=np.float64)[:mol.natoms] for mol in mols])
    return X, n


def get_atomic_kernels_laplacian(mols1, mols2, sigmas):
    """(nsigmas, len(mols1), len(mols2)) local Laplacian kernels."""
    X1, n1 = _stack(mols1)
    X2, n2 = (X1, n1) if mols2 is mols1 else _stack(mols2)
    return get_local_kernels_laplacian(X1, X2, n1, n2, sigmas)


def get_atomic_kernels_gaussian(mols1, mols2, sigmas):
    """(nsigmas, len(mols1), len(mols2)) local Gaussian kernels."""
    X1, n1 = _stack(mols1)
    X2, n2 = (X1, n1) if mols2 is mols1 else _stack(mols2)
    return get_local_kernels_gaussian(X1, X2, n1, n2, sigmas)
