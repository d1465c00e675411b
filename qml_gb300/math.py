"""Drop-ins for qml.math.cho_solve, cho_invert, bkf_solve and bkf_invert
(qml/math.py:33-164, qml/fcho_solve.f90:23-150).

cho_solve solves A x = y with the GPU Cholesky (dpotrf("U") + dpotrs("U")
semantics: the upper triangle of A is read).  Like the reference wrapper it raises
ValueError on shape errors, returns a new x, and leaves A symmetrised from its lower
triangle with the diagonal restored; a non-positive-definite A prints LAPACK's
warning.  cho_invert returns A^-1 like the reference's dpotrf("L") + dpotri("L");
bkf_solve / bkf_invert do the same by Bunch-Kaufman pivoting (dsytrf + dsytrs /
dsytri), so they also take symmetric indefinite matrices.
"""
from __future__ import annotations

import numpy as np
import torch

from . import core


def cho_solve(A, y):
    if len(A.shape) != 2 or A.shape[0] != A.shape[1]:
        raise ValueError('expected square matrix')
    if len(y.shape) != 1 or y.shape[0] != A.shape[1]:
        raise ValueError('expected matrix and vector of same stride size')
    if not torch.cuda.is_available():
        raise RuntimeError("qml_gb300 needs a CUDA device (no CPU fallback)")
    n = A.shape[0]
    # column-major copy: the kernels factor its upper triangle, like dpotrf("U")
    Af = torch.from_numpy(np.asfortranarray(A, dtype=np.float64).T.copy()).cuda()
    yt = torch.from_numpy(np.ascontiguousarray(y, dtype=np.float64)).cuda()
    x, rep = core.solve(Af, yt, 0.0, precision="fp64", max_outer=0, raise_on_info=False)
    if rep["status"] > 0:
        print("WARNING: Error in LAPACK Cholesky decomposition DPOTRF().")
        print("WARNING: The", rep["status"], "-th leading order is not positive definite.")
    # reference wrapper: restore the diagonal, copy the lower triangle to the upper
    if n > 0:
        i_lower = np.tril_indices_from(A)
        A.T[i_lower] = A[i_lower]
    return x.cpu().numpy()


def cho_invert(A, precision="fp64"):
    """Inverse of a symmetric positive-definite matrix (qml/math.py:33-58).

    As in the reference, the result is np.asfortranarray(A): a new array unless A
    already is a Fortran-ordered float64 array, which then receives the inverse in
    place.  A's lower triangle is read (dpotrf("L")); the result is symmetric.  The
    Cholesky factorisation runs in plain FP64 by default, like LAPACK's; with
    precision="mixed" it runs on the tensor cores, several times faster but only
    for well-conditioned matrices: an inverse gets no refinement, so the emulated
    factor's error (~1e-11 relative) is amplified by the condition number.  A matrix
    that is not positive definite prints the reference's warning.
    """
    if len(A.shape) != 2 or A.shape[0] != A.shape[1]:
        raise ValueError('expected square matrix')
    if not torch.cuda.is_available():
        raise RuntimeError("qml_gb300 needs a CUDA device (no CPU fallback)")
    I = np.asfortranarray(A)
    if A.shape[0] == 0:
        return I
    # the rows of this C-ordered array are the columns of I
    At = torch.from_numpy(np.ascontiguousarray(I.T, dtype=np.float64)).cuda()
    Ainv, info = core.cho_invert(At.T, precision=precision)
    if info > 0:
        print("WARNING: Cholesky decomposition DPOTRF() exited with error code:", info)
    I[...] = Ainv.cpu().numpy()
    return I


def bkf_invert(A):
    """Inverse of a symmetric matrix by Bunch-Kaufman pivoting (qml/math.py:100-122):
    the result is np.asfortranarray(A) (in place for a Fortran-ordered float64 A),
    A's lower triangle is read, the result is symmetric."""
    if len(A.shape) != 2 or A.shape[0] != A.shape[1]:
        raise ValueError('expected square matrix')
    if not torch.cuda.is_available():
        raise RuntimeError("qml_gb300 needs a CUDA device (no CPU fallback)")
    I = np.asfortranarray(A)
    if A.shape[0] == 0:
        return I
    At = torch.from_numpy(np.ascontiguousarray(I.T, dtype=np.float64)).cuda()
    Ainv, info = core.bkf_invert(At.T)
    if info > 0:
        print("WARNING: Bunch-Kaufman factorization DSYTRI() exited with error code:", info)
    I[...] = Ainv.cpu().numpy()
    return I


def bkf_solve(A, y):
    """x with A x = y for a symmetric A by Bunch-Kaufman pivoting
    (qml/math.py:125-164).  Raises ValueError on shape errors like the reference,
    returns a new x and leaves A symmetrised from its lower triangle."""
    if len(A.shape) != 2 or A.shape[0] != A.shape[1]:
        raise ValueError('expected square matrix')
    if len(y.shape) != 1 or y.shape[0] != A.shape[1]:
        raise ValueError('expected matrix and vector of same stride size')
    if not torch.cuda.is_available():
        raise RuntimeError("qml_gb300 needs a CUDA device (no CPU fallback)")
    n = A.shape[0]
    Af = torch.from_numpy(np.asfortranarray(A, dtype=np.float64).T.copy()).cuda()
    yt = torch.from_numpy(np.ascontiguousarray(y, dtype=np.float64)).cuda()
    x, info = core.bkf_solve(Af.T, yt)
    if info > 0:
        print("WARNING: Bunch-Kaufman factorization DSYTRI() exited with error code:", info)
    if n > 0:
        i_lower = np.tril_indices_from(A)
        A.T[i_lower] = A[i_lower]
    return x.cpu().numpy()
