"""Minimal drop-in for qml.Compound's XYZ reading and Coulomb matrices
(qml/compound.py:38-105 and :134-216, read_xyz at :296-326)."""
from __future__ import annotations

import numpy as np

from .representations import (NUCLEAR_CHARGE, generate_atomic_coulomb_matrix,
                              generate_coulomb_matrix)


class Compound:
    def __init__(self, xyz=None):
        self.natoms = 0
        self.atomtypes = []
        self.nuclear_charges = np.empty(0, dtype=int)
        self.coordinates = np.empty((0, 3))
        self.representation = np.empty(0)
        self.properties = np.empty(0)
        self.name = None
        if xyz is not None:
            self.read_xyz(xyz)

    def read_xyz(self, filename):
        with open(filename) as f:
            lines = f.readlines()
        self.natoms = int(lines[0])
        self.name = filename
        self.atomtypes = []
        self.nuclear_charges = np.empty(self.natoms, dtype=int)
        self.coordinates = np.empty((self.natoms, 3), dtype=float)
        for i, line in enumerate(lines[2:self.natoms + 2]):
            tokens = line.split()
            if len(tokens) < 4:
                break
            self.atomtypes.append(tokens[0])
            self.nuclear_charges[i] = NUCLEAR_CHARGE[tokens[0]]
            self.coordinates[i] = np.asarray(tokens[1:4], dtype=float)

    def generate_coulomb_matrix(self, size=23, sorting="row-norm"):
        self.representation = generate_coulomb_matrix(self.nuclear_charges, self.coordinates,
                                                      size=size, sorting=sorting)

    def generate_atomic_coulomb_matrix(self, size=23, sorting="row-norm", central_cutoff=1e6,
                                       central_decay=-1, interaction_cutoff=1e6,
                                       interaction_decay=-1, indices=None):
        """Atomic Coulomb matrices of this molecule (note: the method defaults to
        "row-norm" sorting, the module function to "distance", as in the reference)."""
        self.representation = generate_atomic_coulomb_matrix(
            self.nuclear_charges, self.coordinates, size=size, sorting=sorting,
            central_cutoff=central_cutoff, central_decay=central_decay,
            interaction_cutoff=interaction_cutoff, interaction_decay=interaction_decay,
            indices=indices)
