"""bkf_solve / bkf_invert (Bunch-Kaufman pivoting) on the GPU against the reference
tests (tests/test_math.py:74-112) and LAPACK dsytrf + dsytrs / dsytri."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from qml_gb300 import core
from qml_gb300.math import bkf_invert, bkf_solve

pytestmark = pytest.mark.gpu


def test_reference_bkf_solve_and_invert(cuda, oracle):
    g = load_golden("cho_solve_k_local_gaussian.npz")
    A_ref, y_ref = g["A"], g["y"]
    A, y = A_ref.copy(), y_ref.copy()
    x = bkf_solve(A, y)
    assert np.allclose(y, y_ref) and np.allclose(A, A_ref)
    assert np.allclose(x, np.linalg.solve(A_ref, y_ref))
    A = A_ref.copy()
    Ai = bkf_invert(A)
    assert np.allclose(A, A_ref)
    eye = np.eye(A.shape[0])
    assert np.allclose(A @ Ai, eye, atol=1e-7)
    # held to LAPACK's residual on this ill-conditioned matrix
    Ao, _ = oracle.bkf_invert(A_ref)
    assert np.max(np.abs(A @ Ai - eye)) <= 10 * np.max(np.abs(A @ Ao - eye))


def indefinite(n, seed):
    # symmetric, well-conditioned, with eigenvalues of both signs: 2x2 pivots and
    # interchanges happen
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = rng.uniform(0.5, 2.0, n) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    A = (Q * ev) @ Q.T
    return (A + A.T) / 2


@pytest.mark.parametrize("n", [1, 2, 7, 64, 129, 300, 301, 700, 777])
def test_bkf_vs_lapack_indefinite(cuda, oracle, n):
    A = indefinite(n, n)
    y = np.random.default_rng(n + 1).standard_normal(n)
    x = bkf_solve(A.copy(), y.copy())
    xo, info = oracle.bkf_solve(A, y)
    assert info == 0
    assert np.max(np.abs(x - xo)) <= 1e-11 * max(1.0, np.max(np.abs(xo)))
    Ai = bkf_invert(A.copy())
    Ao, _ = oracle.bkf_invert(A)
    assert np.max(np.abs(Ai - Ao)) <= 1e-11 * np.max(np.abs(Ao))
    assert np.array_equal(Ai, Ai.T)


def test_bkf_pivot_cases(cuda, oracle):
    # zero diagonal (forces 2x2 pivots), a swap, and a singular matrix (info)
    A = np.array([[0.0, 1.0, 2.0], [1.0, 0.0, 3.0], [2.0, 3.0, 0.0]])
    y = np.array([1.0, 2.0, 3.0])
    assert np.allclose(bkf_solve(A.copy(), y.copy()), np.linalg.solve(A, y))
    assert np.allclose(bkf_invert(A.copy()), np.linalg.inv(A))
    S = np.zeros((3, 3))
    S[0, 0] = 1.0
    _, info = core.bkf_solve(torch.from_numpy(S).to(cuda), torch.ones(3, dtype=torch.float64,
                                                                      device=cuda))
    assert info == 2
    with pytest.raises(ValueError):
        bkf_solve(np.zeros((3, 3)), np.zeros(4))


@pytest.mark.parametrize("n", [300, 700])
def test_bkf_singular_on_many_ctas(cuda, oracle, n):
    # a zero row/column: the step that meets it is skipped (info), and every CTA must
    # see that decision; the results are the same bits on every run
    rng = np.random.default_rng(n)
    B = rng.standard_normal((n, n))
    j = n // 2
    spd = B @ B.T / n + np.eye(n)
    spd[:, j] = 0.0
    spd[j, :] = 0.0
    sym = B + B.T
    sym[:, n // 3] = 0.0
    sym[n // 3, :] = 0.0
    y = torch.from_numpy(rng.standard_normal(n)).to(cuda)
    for A, info_expected in ((spd, j + 1), (sym, None)):
        At = torch.from_numpy(A).to(cuda)
        runs = [(core.bkf_solve(At, y), core.bkf_invert(At)) for _ in range(3)]
        (x0, si), (a0, vi) = runs[0]
        assert si == vi and si > 0
        if info_expected is not None:
            assert si == info_expected
            assert oracle.bkf_solve(A, y.cpu().numpy())[1] == info_expected
        for (x, s), (ai, v) in runs[1:]:
            assert (s, v) == (si, vi)
            assert torch.equal(x.view(torch.int64), x0.view(torch.int64))
            assert torch.equal(ai.contiguous().view(torch.int64), a0.contiguous().view(torch.int64))


def test_bkf_blocked_on_an_ill_conditioned_kernel_matrix(cuda, oracle):
    # a Gaussian kernel matrix (condition ~1e5) above the blocked threshold, several
    # panels: the solve (emulated trailing updates) and the inverse (FP64 ones) keep
    # LAPACK's residuals
    rng = np.random.default_rng(3)
    n = 1500
    X = rng.standard_normal((n, 20))
    D2 = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    K = np.exp(-D2 / (2 * 4.0 ** 2)) + 1e-8 * np.eye(n)
    y = rng.standard_normal(n)
    x = bkf_solve(K.copy(), y.copy())
    xo, info = oracle.bkf_solve(K, y)
    assert info == 0
    assert np.max(np.abs(K @ x - y)) <= 10 * np.max(np.abs(K @ xo - y))
    Ki = bkf_invert(K.copy())
    Ko, _ = oracle.bkf_invert(K)
    eye = np.eye(n)
    assert np.max(np.abs(K @ Ki - eye)) <= 10 * np.max(np.abs(K @ Ko - eye))


def test_bkf_solve_above_the_shared_memory_ring(cuda, oracle):
    # n = 6000: the solve's L columns no longer fit the shared-memory ring, so dsytrs
    # reads them straight from the transposed copy; held to LAPACK's residual
    rng = np.random.default_rng(6000)
    n = 6000
    B = rng.standard_normal((n, n))
    A = B + B.T
    y = rng.standard_normal(n)
    x = bkf_solve(A.copy(), y.copy())
    xo, info = oracle.bkf_solve(A, y)
    assert info == 0
    assert np.max(np.abs(A @ x - y)) <= 10 * np.max(np.abs(A @ xo - y))


@pytest.mark.parametrize("n", [600])
def test_bkf_blocked_with_2x2_pivots_everywhere(cuda, oracle, n):
    # a zero diagonal makes almost every pivot 2x2, including the ones that end a
    # panel one column late; solve and inverse held to LAPACK
    rng = np.random.default_rng(n + 7)
    B = rng.standard_normal((n, n))
    A = B + B.T
    np.fill_diagonal(A, 0.0)
    y = rng.standard_normal(n)
    x = bkf_solve(A.copy(), y.copy())
    xo, info = oracle.bkf_solve(A, y)
    assert info == 0
    assert np.max(np.abs(A @ x - y)) <= 10 * np.max(np.abs(A @ xo - y))
    Ai = bkf_invert(A.copy())
    Ao, _ = oracle.bkf_invert(A)
    eye = np.eye(n)
    assert np.max(np.abs(A @ Ai - eye)) <= 10 * np.max(np.abs(A @ Ao - eye))
