"""Batched XYZ ingestion to the device and KRR model persistence.

The reference reads one XYZ file per Compound (qml/compound.py:296-326) and keeps
models only in memory.  Here the library's native parser reads many files on host
threads into one ragged MoleculeBatch, which moves to the device in one pinned copy per array and feeds the
batched Coulomb-matrix kernel; a fitted KRR model (hyper-parameters, training
representations, alpha) saves to and loads from one .npz file, so a serving process
can restart without refitting.
"""
from __future__ import annotations

import ctypes
import os
from typing import Iterable, Sequence

import numpy as np
import torch

from . import _lib
from .krr import KRR, molecules_to_device
from .representations import NUCLEAR_CHARGE
from .synthetic import MoleculeBatch

FORMAT = 1


def read_xyz(path: str):
    """(charges float64 (natoms,), coordinates float64 (natoms, 3)) of one XYZ file,
    parsed like Compound.read_xyz: the atom count on line 1, atoms from line 3 on,
    stopping early at a line with fewer than four fields."""
    with open(path) as f:
        lines = f.readlines()
    natoms = int(lines[0])
    z = np.empty(natoms, dtype=np.float64)
    r = np.empty((natoms, 3), dtype=np.float64)
    n = 0
    for line in lines[2:natoms + 2]:
        t = line.split()
        if len(t) < 4:
            break
        z[n] = NUCLEAR_CHARGE[t[0]]
        r[n] = [float(v) for v in t[1:4]]
        n += 1
    return z[:n], r[:n]


def read_xyz_batch(paths: Sequence[str], workers: int = 0) -> MoleculeBatch:
    """Parse many XYZ files into one ragged batch (input order kept).

    qmlg_read_files reads the files and qmlg_parse_xyz parses them, both on `workers`
    host threads (0 = one per hardware thread).  A file that parser does not accept
    (non-ASCII text, a number Python reads but strtod does not) is parsed by
    read_xyz instead, which also raises the reference's error for a malformed file."""
    paths = list(paths)
    nf = len(paths)
    lib = _lib.load()
    workers = int(workers)
    names = (ctypes.c_char_p * max(nf, 1))(*[os.fsencode(p) for p in paths])
    sizes = np.empty(nf, dtype=np.int64)
    _lib.check(lib.qmlg_read_files(names, nf, workers, sizes.ctypes.data, None, None, None),
               "qmlg_read_files")
    # an unreadable file gets no bytes: the parser then flags it, and read_xyz
    # raises the reference's error for it
    starts = np.zeros(nf + 1, dtype=np.int64)
    starts[1:] = np.cumsum(np.maximum(sizes, 0))
    text = np.empty(max(int(starts[-1]), 1), dtype=np.uint8)
    unread = np.zeros(nf, dtype=np.int32)
    _lib.check(lib.qmlg_read_files(names, nf, workers, sizes.ctypes.data, text.ctypes.data,
                                   starts.ctypes.data, unread.ctypes.data), "qmlg_read_files")
    body = text[:int(starts[-1])]
    cap = int(np.count_nonzero(body == 10)) + int(np.count_nonzero(body == 13)) + nf
    charges = np.empty(cap, dtype=np.float64)
    coords = np.empty((cap, 3), dtype=np.float64)
    offsets = np.empty(nf + 1, dtype=np.int64)
    status = np.empty(nf, dtype=np.int32)
    _lib.check(lib.qmlg_parse_xyz(text.ctypes.data, starts.ctypes.data, nf, workers,
                                  offsets.ctypes.data, status.ctypes.data, charges.ctypes.data,
                                  coords.ctypes.data, cap), "qmlg_parse_xyz")
    status |= unread
    if status.any():
        mols = [read_xyz(paths[f]) if status[f] else
                (charges[offsets[f]:offsets[f + 1]], coords[offsets[f]:offsets[f + 1]])
                for f in range(nf)]
        counts = np.array([z.shape[0] for z, _ in mols], dtype=np.int64)
        offsets = np.zeros(nf + 1, dtype=np.int64)
        offsets[1:] = np.cumsum(counts)
        charges = np.concatenate([z for z, _ in mols])
        coords = np.concatenate([r for _, r in mols]).reshape(-1, 3)
    total = int(offsets[-1])
    return MoleculeBatch(charges[:total].copy(), coords[:total].copy(), offsets, np.zeros(nf))


def xyz_to_device(paths: Iterable[str], device="cuda", workers: int = 0):
    """(charges, coordinates, offsets) CUDA tensors of many XYZ files: ready for
    core.coulomb_matrix_batch / atomic_coulomb_matrix_batch."""
    return molecules_to_device(read_xyz_batch(list(paths), workers), device=device)


def save_krr(path: str, model: KRR) -> None:
    """Write a fitted KRR model to one .npz file."""
    if model.alpha is None or model.X is None:
        raise RuntimeError("fit() first")
    np.savez(path, format=FORMAT, kernel=model.kernel, sigma=model.sigma, lam=model.lam,
             precision=model.precision, max_outer=model.max_outer, tol=model.tol,
             X=model.X.detach().cpu().numpy(), alpha=model.alpha.detach().cpu().numpy())


def load_krr(path: str, device="cuda") -> KRR:
    """Read a model written by save_krr, its tensors on `device`."""
    with np.load(path, allow_pickle=False) as f:
        if int(f["format"]) != FORMAT:
            raise ValueError("unknown model file format %d" % int(f["format"]))
        m = KRR(kernel=str(f["kernel"]), sigma=float(f["sigma"]), lam=float(f["lam"]),
                precision=str(f["precision"]), max_outer=int(f["max_outer"]), tol=float(f["tol"]))
        m.X = torch.from_numpy(f["X"].copy()).to(device)
        m.alpha = torch.from_numpy(f["alpha"].copy()).to(device)
    return m
