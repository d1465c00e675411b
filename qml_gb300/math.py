"""Drop-in for qml.math.cho_solve (qml/math.py:60-97, qml/fcho_solve.f90:23-52).

Solves A x = y with the GPU Cholesky (dpotrf("U") + dpotrs("U") semantics: the
upper triangle of A is read).  Like the reference wrapper it raises ValueError on
shape errors, returns a new x, and leaves A symmetrised from its lower triangle
with the diagonal restored; a non-positive-definite A prints LAPACK's warning.
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
