"""cho_invert on the GPU (the Schur complement of the augmented matrix) against
the reference test (tests/test_math.py:54-71) and LAPACK dpotrf + dpotri."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from qml_gb300 import core
from qml_gb300.math import cho_invert

pytestmark = pytest.mark.gpu


def test_reference_cho_invert(cuda, oracle):
    # the default (plain FP64 factorisation, as LAPACK's); the tensor-core one is not
    # accurate enough for an unrefined inverse of this ill-conditioned matrix
    A_ref = load_golden("cho_solve_k_local_gaussian.npz")["A"]
    A = A_ref.copy()
    Ai = cho_invert(A)
    assert np.array_equal(A, A_ref)                     # A is unchanged
    assert np.allclose(A @ Ai, np.eye(A.shape[0]), atol=1e-7)
    assert np.array_equal(Ai, Ai.T)
    # this matrix is ill-conditioned (two FP64 inverses differ by ~cond * u), so the
    # inverse is held to LAPACK's residual rather than to LAPACK's digits
    Ao = oracle.cho_invert(A_ref)
    eye = np.eye(A.shape[0])
    assert np.max(np.abs(A @ Ai - eye)) <= 10 * np.max(np.abs(A @ Ao - eye))


@pytest.mark.parametrize("n", [1, 63, 130, 700])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cho_invert_vs_lapack(cuda, oracle, n, precision):
    # a well-conditioned SPD matrix: agreement at the FP64 rounding level
    rng = np.random.default_rng(n)
    B = rng.standard_normal((n, n))
    A = B @ B.T / n + np.eye(n)
    Ai = cho_invert(A.copy(), precision=precision)
    Ao = oracle.cho_invert(A)
    assert np.max(np.abs(Ai - Ao)) <= 1e-12 * np.max(np.abs(Ao))


def test_cho_invert_reads_lower_triangle_and_fortran_in_place(cuda, oracle):
    rng = np.random.default_rng(3)
    n = 90
    B = rng.standard_normal((n, n))
    A = B @ B.T / n + np.eye(n)
    junk = A.copy()
    junk[np.triu_indices(n, 1)] = 7.0          # only the lower triangle is read
    F = np.asfortranarray(junk)
    out = cho_invert(F)
    assert out is F                             # Fortran-ordered float64: in place
    assert np.max(np.abs(out - oracle.cho_invert(A))) <= 1e-12 * np.max(np.abs(out))


def test_cho_invert_not_positive_definite(cuda, capsys):
    A = np.diag([1.0, 2.0, -1.0, 4.0])
    cho_invert(A, precision="fp64")
    assert "exited with error code: 3" in capsys.readouterr().out
    At = torch.from_numpy(A).to(cuda)
    _, info = core.cho_invert(At, precision="mixed")
    assert info == 3
    with pytest.raises(ValueError):
        cho_invert(np.zeros((3, 4)))
