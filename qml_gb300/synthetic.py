"""Seeded synthetic molecules that stand in for QM7-like data.

QM7 (7101 molecules, at most 23 atoms of H/C/N/O/S) is the data set the reference's
KRR tests and tutorial use (``tests/test_energy_krr_cmat.py:54-113``,
``docs/source/tutorial.rst:84-166``).  The generator below draws molecules with the
same shape so that the sorted Coulomb matrix has size 23 (276 features):

* ``n_atoms ~ U{5..23}``;
* ``Z`` from {1, 6, 7, 8, 16} with probabilities {0.5, 0.35, 0.07, 0.07, 0.01};
* coordinates by a random walk: each new atom sits ``U(1.0, 1.6)`` Angstrom from a
  uniformly chosen earlier atom in a uniformly random direction, and is rejected
  (and re-drawn) if it lands within 0.9 Angstrom of any atom already placed;
* labels ``y = 0.01 * sum_{i<j} Z_i Z_j / r_ij + N(0, 1)`` in FP64.

The draw is vectorised over molecules (one placement round per atom index), so a
given seed reproduces the same molecules on any machine with the same numpy.
Molecules are returned in ragged form: flat charges and coordinates plus an offsets
array (``offsets[m]:offsets[m+1]`` are molecule ``m``'s atoms).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ELEMENTS = np.array([1, 6, 7, 8, 16], dtype=np.int32)
ELEMENT_P = np.array([0.5, 0.35, 0.07, 0.07, 0.01])
MAX_ATOMS = 23


@dataclass
class MoleculeBatch:
    """Ragged batch of molecules (host arrays)."""

    charges: np.ndarray      # (total_atoms,) float64 nuclear charges
    coordinates: np.ndarray  # (total_atoms, 3) float64, Angstrom
    offsets: np.ndarray      # (n_mol + 1,) int64
    labels: np.ndarray       # (n_mol,) float64

    @property
    def n_mol(self) -> int:
        return int(self.offsets.shape[0] - 1)

    def molecule(self, m: int):
        a, b = int(self.offsets[m]), int(self.offsets[m + 1])
        return self.charges[a:b], self.coordinates[a:b]

    def slice(self, start: int, stop: int) -> "MoleculeBatch":
        a, b = int(self.offsets[start]), int(self.offsets[stop])
        return MoleculeBatch(self.charges[a:b].copy(), self.coordinates[a:b].copy(),
                             (self.offsets[start:stop + 1] - a).copy(),
                             self.labels[start:stop].copy())


def generate_molecules(n_mol: int, seed: int = 0, max_atoms: int = MAX_ATOMS,
                       min_atoms: int = 5) -> MoleculeBatch:
    """Draw ``n_mol`` random-walk molecules with the QM7-like distribution above."""
    rng = np.random.default_rng(seed)
    n_atoms = rng.integers(min_atoms, max_atoms + 1, size=n_mol)
    z = ELEMENTS[rng.choice(len(ELEMENTS), size=(n_mol, max_atoms), p=ELEMENT_P)]
    pos = np.zeros((n_mol, max_atoms, 3))
    for a in range(1, max_atoms):
        todo = np.nonzero(n_atoms > a)[0]
        for _ in range(10000):
            if todo.size == 0:
                break
            parent = rng.integers(0, a, size=todo.size)
            v = rng.normal(size=(todo.size, 3))
            v /= np.linalg.norm(v, axis=1, keepdims=True)
            dist = rng.uniform(1.0, 1.6, size=todo.size)
            cand = pos[todo, parent] + dist[:, None] * v
            d2 = np.sum((pos[todo, :a] - cand[:, None, :]) ** 2, axis=2)
            ok = np.min(d2, axis=1) >= 0.81
            pos[todo[ok], a] = cand[ok]
            todo = todo[~ok]
        else:  # pragma: no cover - the walk always finds room in practice
            raise RuntimeError("random-walk placement did not converge")

    offsets = np.zeros(n_mol + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(n_atoms)
    mask = np.arange(max_atoms)[None, :] < n_atoms[:, None]
    charges = z[mask].astype(np.float64)
    coords = pos[mask]

    # labels: 0.01 * sum_{i<j} Z_i Z_j / r_ij + N(0, 1), in chunks of molecules
    iu = np.triu(np.ones((max_atoms, max_atoms), dtype=bool), 1)
    energy = np.empty(n_mol)
    for a in range(0, n_mol, 4096):
        b = min(n_mol, a + 4096)
        diff = pos[a:b, :, None, :] - pos[a:b, None, :, :]
        r = np.sqrt(np.sum(diff * diff, axis=3))
        zz = z[a:b, :, None].astype(np.float64) * z[a:b, None, :]
        pair = mask[a:b, :, None] & mask[a:b, None, :] & iu[None]
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.where(pair, zz / np.where(pair, r, 1.0), 0.0)
        energy[a:b] = e.sum(axis=(1, 2))
    labels = 0.01 * energy + rng.normal(size=n_mol)
    return MoleculeBatch(charges, coords, offsets, labels)


def padded(batch: MoleculeBatch, max_atoms: int = MAX_ATOMS):
    """Padded (n_mol, max_atoms) charges and (n_mol, max_atoms, 3) coordinates."""
    n = batch.n_mol
    counts = np.diff(batch.offsets)
    z = np.zeros((n, max_atoms))
    r = np.zeros((n, max_atoms, 3))
    mask = np.arange(max_atoms)[None, :] < counts[:, None]
    z[mask] = batch.charges
    r[mask] = batch.coordinates
    return z, r, counts
