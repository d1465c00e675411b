"""Batched XYZ ingestion to the device and KRR model persistence.

The reference reads one XYZ file per Compound (qml/compound.py:296-326) and keeps
models only in memory.  Here many files are parsed in parallel into one ragged
MoleculeBatch, which moves to the device in one pinned copy per array and feeds the
batched Coulomb-matrix kernel; a fitted KRR model (hyper-parameters, training
representations, alpha) saves to and loads from one .npz file, so a serving process
can restart without refitting.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
from typing import Iterable, List, Sequence

import numpy as np
import torch

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
    """Parse many XYZ files (in parallel, input order kept) into one ragged batch."""
    paths = list(paths)
    workers = workers or min(32, (os.cpu_count() or 1))
    if len(paths) > 64 and workers > 1:
        with cf.ThreadPoolExecutor(workers) as ex:
            mols = list(ex.map(read_xyz, paths, chunksize=64))
    else:
        mols = [read_xyz(p) for p in paths]
    counts = np.array([z.shape[0] for z, _ in mols], dtype=np.int64)
    offsets = np.zeros(len(mols) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(counts)
    charges = np.concatenate([z for z, _ in mols]) if mols else np.empty(0)
    coords = np.concatenate([r for _, r in mols]) if mols else np.empty((0, 3))
    return MoleculeBatch(charges, coords.reshape(-1, 3), offsets, np.zeros(len(mols)))


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
