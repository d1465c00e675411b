"""Drop-ins for qml.representations.generate_coulomb_matrix (qml/representations.py:69-119)
and generate_atomic_coulomb_matrix (:121-230).

Same names, arguments, output shapes and error behaviour as the reference; the
matrices are computed by the CUDA kernels behind qmlg_coulomb_matrix and
qmlg_atomic_coulomb_matrix.  The batched forms (``generate_coulomb_matrix_batch``,
``generate_atomic_coulomb_matrix_batch``) are the performance path: one launch for
a whole ragged batch instead of one call per molecule.
"""
from __future__ import annotations

import numpy as np
import torch

from . import core

# element symbol -> nuclear charge, the table of qml/data.py:23 (elements 1-112, then
# the placeholder names Uuq = 114 and Uuh = 116)
_SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn "
            "Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce "
            "Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn "
            "Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf Db Sg Bh Hs Mt Ds Rg Cn")
NUCLEAR_CHARGE = {s: z for z, s in enumerate(_SYMBOLS.split(), start=1)}
NUCLEAR_CHARGE.update(Uuq=114, Uuh=116)


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("qml_gb300 needs a CUDA device (no CPU fallback)")
    return torch.device("cuda")


def generate_coulomb_matrix(nuclear_charges, coordinates, size=23, sorting="row-norm"):
    """Coulomb matrix of one molecule, shape (size*(size+1)//2,), float64.

    sorting="row-norm" orders atoms by descending row 2-norm (ties: higher input
    index first, as the reference's repeated minloc does); "unsorted" keeps input
    order.  Unknown sorting prints the reference's message and raises SystemExit;
    a charges/coordinates length mismatch does the same, like the Fortran ``stop``.
    """
    if sorting not in ("row-norm", "unsorted"):
        print("ERROR: Unknown sorting scheme requested")
        raise SystemExit
    z = np.asarray(nuclear_charges, dtype=np.float64).reshape(-1)
    r = np.asarray(coordinates, dtype=np.float64).reshape(-1, 3)
    if r.shape[0] != z.shape[0]:
        print("ERROR: Coulomb matrix generation")
        print(r.shape[0], "coordinates, but", z.shape[0], "atom_types!")
        raise SystemExit
    if z.shape[0] > size:
        raise ValueError("molecule has %d atoms but size=%d" % (z.shape[0], size))
    dev = _device()
    offsets = torch.tensor([0, z.shape[0]], dtype=torch.int64, device=dev)
    out = core.coulomb_matrix_batch(torch.from_numpy(z).to(dev), torch.from_numpy(r).to(dev),
                                    offsets, size=size, sorting=sorting)
    return out[0].cpu().numpy()


def generate_coulomb_matrix_batch(charges, coordinates, offsets, size=23, sorting="row-norm"):
    """Coulomb matrices of a ragged batch.  Accepts numpy arrays or CUDA tensors;
    returns a CUDA tensor (n_mol, size*(size+1)//2)."""
    dev = _device()

    def dev_t(a, dtype):
        if isinstance(a, torch.Tensor):
            return a.to(device=dev, dtype=dtype)
        return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)

    return core.coulomb_matrix_batch(dev_t(charges, torch.float64),
                                     dev_t(coordinates, torch.float64).reshape(-1, 3),
                                     dev_t(offsets, torch.int64), size=size, sorting=sorting)


def generate_atomic_coulomb_matrix(nuclear_charges, coordinates, size=23, sorting="distance",
                                   central_cutoff=1e6, central_decay=-1, interaction_cutoff=1e6,
                                   interaction_decay=-1, indices=None):
    """Atomic Coulomb matrices of one molecule, shape (n_central, size*(size+1)//2).

    One row per central atom: every atom (indices=None), the listed 0-based
    indices, or every atom of one element (indices="C", say; none present gives
    np.zeros((0, 0))).  sorting "row-norm" orders the atoms by descending row norm
    with the central atom first, "distance" by distance to the central atom; the
    soft cutoffs mask the matrix as in the reference.  Unknown sorting or element
    strings print the reference's message and raise SystemExit; a molecule with more
    than `size` atoms inside the central cutoff raises QmlgError (the reference stops).
    """
    z = np.asarray(nuclear_charges, dtype=np.float64).reshape(-1)
    r = np.asarray(coordinates, dtype=np.float64).reshape(-1, 3)
    if indices is None:
        central = np.arange(z.shape[0])
    elif isinstance(indices, str):
        if indices in NUCLEAR_CHARGE:
            central = np.where(z == NUCLEAR_CHARGE[indices])[0]
            if central.size == 0:
                return np.zeros((0, 0))
        else:
            print("ERROR: Unknown value %s given for 'indices' variable" % indices)
            raise SystemExit
    else:
        central = np.asarray(indices, dtype=int).reshape(-1)
    if sorting not in ("row-norm", "distance"):
        print("ERROR: Unknown sorting scheme requested")
        raise SystemExit
    if r.shape[0] != z.shape[0]:
        print("ERROR: Coulomb matrix generation")
        print(r.shape[0], "coordinates, but", z.shape[0], "atom_types!")
        raise SystemExit
    dev = _device()
    out = core.atomic_coulomb_matrix_batch(
        torch.from_numpy(z).to(dev), torch.from_numpy(r).to(dev),
        torch.tensor([0, z.shape[0]], dtype=torch.int64, device=dev), size=size, sorting=sorting,
        central_cutoff=central_cutoff, central_decay=central_decay,
        interaction_cutoff=interaction_cutoff, interaction_decay=interaction_decay,
        central_offsets=torch.tensor([0, central.shape[0]], dtype=torch.int64, device=dev),
        central_atoms=torch.from_numpy(central.astype(np.int32)).to(dev))
    return out.cpu().numpy()


def generate_atomic_coulomb_matrix_batch(charges, coordinates, offsets, size=23,
                                         sorting="distance", **cutoffs):
    """Atomic Coulomb matrices of a ragged batch, every atom central: a CUDA tensor
    (total_atoms, size*(size+1)//2), rows in atom order.  cutoffs: central_cutoff,
    central_decay, interaction_cutoff, interaction_decay as above."""
    dev = _device()

    def dev_t(a, dtype):
        if isinstance(a, torch.Tensor):
            return a.to(device=dev, dtype=dtype)
        return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)

    return core.atomic_coulomb_matrix_batch(dev_t(charges, torch.float64),
                                            dev_t(coordinates, torch.float64).reshape(-1, 3),
                                            dev_t(offsets, torch.int64), size=size,
                                            sorting=sorting, **cutoffs)
