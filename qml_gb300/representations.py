"""Drop-in for qml.representations.generate_coulomb_matrix (qml/representations.py:69-119).

Same name, arguments, output shape and error behaviour as the reference; the
matrix is computed by the CUDA kernel behind qmlg_coulomb_matrix.  The batched
form (``generate_coulomb_matrix_batch``) is the performance path: one launch for
a whole ragged batch instead of one call per molecule.
"""
from __future__ import annotations

import numpy as np
import torch

from . import core


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
