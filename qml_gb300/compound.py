"""Minimal drop-in for qml.Compound's XYZ reading and Coulomb matrix
(qml/compound.py:38-105, read_xyz at :296-326)."""
from __future__ import annotations

import numpy as np

from .representations import generate_coulomb_matrix

NUCLEAR_CHARGE = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9,
                  "Ne": 10, "Na": 11, "Mg": 12, "Al": 13, "Si": 14, "P": 15, "S": 16, "Cl": 17,
                  "Ar": 18, "K": 19, "Ca": 20, "Br": 35, "I": 53}


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
