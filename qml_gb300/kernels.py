"""Drop-ins for qml.kernels.gaussian_kernel / laplacian_kernel (qml/kernels.py:36-92).

Host arrays in, a Fortran-ordered (na, nb) float64 ndarray out, exactly like the
reference; the matrix is computed on the GPU (qmlg_gaussian_kernel /
qmlg_laplacian_kernel).  When B is A the symmetric kernel computes one triangle
and mirrors it, so K is exactly symmetric.
"""
from __future__ import annotations

import numpy as np
import torch

from . import core


def _to_dev(X):
    if not torch.cuda.is_available():
        raise RuntimeError("qml_gb300 needs a CUDA device (no CPU fallback)")
    return torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).cuda()


def _kernel(kind, A, B, sigma):
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    same = B is A or (A.shape == B.shape and np.shares_memory(A, B) and np.array_equal(A, B))
    At = _to_dev(A)
    Bt = At if same else _to_dev(B)
    K = core.kernel_matrix(kind, At, Bt, sigma, symmetric=same)
    # K is a Fortran-ordered (na, nb) view; K.T is C-contiguous (nb, na)
    return np.asfortranarray(K.T.cpu().numpy().T)


def laplacian_kernel(A, B, sigma):
    """K_ij = exp(-|A_i - B_j|_1 / sigma), shape (na, nb), order='F'."""
    return _kernel("laplacian", A, B, sigma)


def gaussian_kernel(A, B, sigma):
    """K_ij = exp(-|A_i - B_j|_2^2 / (2 sigma^2)), shape (na, nb), order='F'."""
    return _kernel("gaussian", A, B, sigma)
