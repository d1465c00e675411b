"""Drop-ins for qml.kernels (qml/kernels.py:36-299): gaussian_kernel,
laplacian_kernel, linear_kernel, sargan_kernel, matern_kernel and the local kernels
get_local_kernels_gaussian / get_local_kernels_laplacian.

Host arrays in, a Fortran-ordered (na, nb) float64 ndarray out, exactly like the
reference; the matrix is computed on the GPU (qmlg_gaussian_kernel,
qmlg_laplacian_kernel, qmlg_linear_kernel, qmlg_sargan_kernel,
qmlg_matern_kernel_l2).  When B is A the symmetric kernel computes one triangle
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


def _kernel(kind, A, B, sigma, **kw):
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    same = B is A or (A.shape == B.shape and np.shares_memory(A, B) and np.array_equal(A, B))
    At = _to_dev(A)
    Bt = At if same else _to_dev(B)
    K = core.kernel_matrix(kind, At, Bt, sigma, symmetric=same, **kw)
    # K is a Fortran-ordered (na, nb) view; K.T is C-contiguous (nb, na)
    return np.asfortranarray(K.T.cpu().numpy().T)


def laplacian_kernel(A, B, sigma):
    """K_ij = exp(-|A_i - B_j|_1 / sigma), shape (na, nb), order='F'."""
    return _kernel("laplacian", A, B, sigma)


def gaussian_kernel(A, B, sigma):
    """K_ij = exp(-|A_i - B_j|_2^2 / (2 sigma^2)), shape (na, nb), order='F'."""
    return _kernel("gaussian", A, B, sigma)


def linear_kernel(A, B):
    """K_ij = A_i . B_j, shape (na, nb), order='F' (qml/kernels.py:94-120)."""
    return _kernel("linear", A, B, 1.0)


def sargan_kernel(A, B, sigma, gammas):
    """K_ij = exp(-|A_i - B_j|_1 / sigma) (1 + sum_k gamma_k |A_i - B_j|_1^k / sigma^k)
    (qml/kernels.py:122-156); no gammas gives the Laplacian kernel, as there."""
    gammas = np.asarray(gammas, dtype=np.float64).reshape(-1)
    if len(gammas) == 0:
        return laplacian_kernel(A, B, sigma)
    return _kernel("sargan", A, B, sigma, gammas=torch.from_numpy(gammas))


def matern_kernel(A, B, sigma, order=0, metric="l1"):
    """Matern kernel of order 0, 1 or 2 with the L1 or L2 distance
    (qml/kernels.py:158-215).  L1 goes through the Sargan kernel with the reference's
    gammas and rescaled sigma; unknown orders and metrics print the reference's message
    and raise SystemExit."""
    if metric == "l1":
        if order == 0:
            gammas = []
        elif order == 1:
            gammas = [1]
            sigma /= np.sqrt(3)
        elif order == 2:
            gammas = [1, 1 / 3.0]
            sigma /= np.sqrt(5)
        else:
            print("Order:%d not implemented in Matern Kernel" % order)
            raise SystemExit
        return sargan_kernel(A, B, sigma, gammas)
    elif metric == "l2":
        pass
    else:
        print("Error: Unknown distance metric %s in Matern kernel" % str(metric))
        raise SystemExit
    # the reference's Fortran takes every order other than 0 and 1 as order 2
    return _kernel("matern_l2", A, B, sigma, order=order if order in (0, 1) else 2)


def _local(kind, A, B, na, nb, sigmas):
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    assert np.sum(na) == A.shape[0], "Error in A input"
    assert np.sum(nb) == B.shape[0], "Error in B input"
    assert A.shape[1] == B.shape[1], "Error in representation sizes"
    same = B is A or (A.shape == B.shape and np.shares_memory(A, B) and np.array_equal(A, B))
    na = np.asarray(na, dtype=np.int64).reshape(-1)
    nb = np.asarray(nb, dtype=np.int64).reshape(-1)
    same = same and np.array_equal(na, nb)
    At = _to_dev(A)
    Bt = At if same else _to_dev(B)
    oa = torch.from_numpy(np.concatenate([[0], np.cumsum(na)]).astype(np.int64))
    ob = torch.from_numpy(np.concatenate([[0], np.cumsum(nb)]).astype(np.int64))
    K = core.local_kernels(kind, At, Bt, oa, ob, np.asarray(sigmas, dtype=np.float64),
                           symmetric=same)
    return np.asfortranarray(K.cpu().numpy())


def get_local_kernels_gaussian(A, B, na, nb, sigmas):
    """K[s, i, j] = sum_{a in i} sum_{b in j} exp(-|A_a - B_b|_2^2 / (2 sigma_s^2)),
    shape (nsigmas, len(na), len(nb)); atom rows concatenated by molecule
    (qml/kernels.py:218-257)."""
    return _local("gaussian", A, B, na, nb, sigmas)


def get_local_kernels_laplacian(A, B, na, nb, sigmas):
    """K[s, i, j] = sum_{a in i} sum_{b in j} exp(-|A_a - B_b|_1 / sigma_s)
    (qml/kernels.py:259-299)."""
    return _local("laplacian", A, B, na, nb, sigmas)
