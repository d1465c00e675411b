"""Cholesky solve on the GPU: LAPACK semantics (plain FP64) and the mixed path
(emulated-FP64 tensor-core factor + refinement on the exact residual) against the
oracle.
The mixed path's bar is <= 1e-8 relative error on alpha against the refined
oracle solution for the same FP64 K."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from qml_gb300 import core
from qml_gb300.math import cho_solve
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_reference_cho_solve(cuda, oracle):
    # tests/test_math.py:32-52 through the drop-in
    g = load_golden("cho_solve_k_local_gaussian.npz")
    A, y = g["A"].copy(), g["y"].copy()
    x = cho_solve(A, y)
    assert np.allclose(y, g["y"]) and np.allclose(A, g["A"])
    assert np.allclose(x, np.linalg.solve(g["A"], g["y"]))
    xr = oracle.refined_solve(g["A"], g["y"], 0.0)
    assert rel(x, xr) < 1e-5  # cond(A) ~ 4e9: FP64 forward error


def test_cho_solve_shape_errors(cuda):
    with pytest.raises(ValueError):
        cho_solve(np.eye(3)[:2], np.ones(3))
    with pytest.raises(ValueError):
        cho_solve(np.eye(3), np.ones(2))


def test_cho_solve_symmetrises_from_lower(cuda, oracle):
    rng = np.random.default_rng(1)
    M = rng.normal(size=(70, 70))
    S = M @ M.T + 70 * np.eye(70)
    A = S.copy()
    A[np.triu_indices(70, 1)] = 0.0  # only the lower triangle is meaningful ...
    A_upper = S.copy()  # ... but dpotrf("U") reads the upper one
    x = cho_solve(A_upper, np.ones(70))
    assert rel(x, np.linalg.solve(S, np.ones(70))) < 1e-12
    cho_solve(A, np.ones(70))  # reads the (diagonal-only) upper triangle
    assert np.array_equal(A, np.tril(S) + np.tril(S, -1).T)


@pytest.fixture(scope="module")
def krr_system(oracle):
    b = generate_molecules(1500, seed=13)
    X = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    return X, b.labels


@pytest.mark.parametrize("n", [1, 63, 64, 100, 1500])
def test_fp64_solve_matches_lapack(cuda, oracle, krr_system, n):
    X, y = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:n], X[:n], 1000.0))
    lam = 1e-4
    Kt = torch.from_numpy(K).to(cuda)
    x, rep = core.solve(Kt.clone(), torch.from_numpy(y[:n]).to(cuda), lam, precision="fp64",
                        max_outer=0)
    x = x.cpu().numpy()
    xl = oracle.cho_solve(K + lam * np.eye(n), y[:n])
    xr = oracle.refined_solve(K, y[:n], lam)
    # same algorithm class as LAPACK: forward error of the order cond * u
    assert rel(x, xr) < 1e-5 and rel(xl, xr) < 1e-5
    # with refinement on the exact residual: agrees with the refined oracle to <= 1e-12
    x2, rep2 = core.solve(Kt.clone(), torch.from_numpy(y[:n]).to(cuda), lam, precision="fp64",
                          max_outer=10)
    assert rel(x2.cpu().numpy(), xr) < 1e-12


def test_factor_matches_lapack_upper(cuda, oracle, krr_system):
    from scipy.linalg import lapack
    X, _ = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:300], X[:300], 1000.0)) + 1e-3 * np.eye(300)
    Kt = torch.from_numpy(np.asfortranarray(K)).to(cuda)  # as the column-major matrix
    KtF = torch.from_numpy(np.ascontiguousarray(K.T)).to(cuda)
    assert core.cholesky(KtF) == 0
    U = KtF.cpu().numpy().T  # column-major view back
    c, info = lapack.dpotrf(np.asfortranarray(K), lower=0, clean=1)
    assert info == 0
    assert np.max(np.abs(np.triu(U) - c)) < 1e-10 * np.max(np.abs(c))
    assert np.array_equal(np.tril(U, -1), np.tril(K, -1))  # other triangle untouched
    del Kt


def test_not_positive_definite_info(cuda, oracle):
    from scipy.linalg import lapack
    rng = np.random.default_rng(2)
    M = rng.normal(size=(150, 150))
    S = M @ M.T + np.eye(150)
    S[100, 100] = -5.0
    _, info = lapack.dpotrf(np.asfortranarray(S), lower=0)
    assert info > 0
    St = torch.from_numpy(np.ascontiguousarray(S.T)).to(cuda)
    assert core.cholesky(St) == info
    _, rep = core.solve(torch.from_numpy(S).to(cuda), torch.ones(150, dtype=torch.float64,
                        device=cuda), 0.0, precision="fp64", raise_on_info=False)
    assert rep["status"] == info


@pytest.mark.parametrize("lam", [1e-4, 1e-6, 1e-8])
def test_mixed_solve_1e8(cuda, oracle, krr_system, lam):
    X, y = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X, X, 1000.0))
    xr = oracle.refined_solve(K, y, lam)
    x, rep = core.solve(torch.from_numpy(K).to(cuda), torch.from_numpy(y).to(cuda), lam,
                        precision="mixed")
    assert rep["status"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-8, rep


def test_mixed_solve_deterministic(cuda, oracle, krr_system):
    X, y = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:700], X[:700], 500.0))
    runs = [core.solve(torch.from_numpy(K).to(cuda), torch.from_numpy(y[:700]).to(cuda), 1e-6,
                       precision="mixed")[0].cpu().numpy() for _ in range(2)]
    assert np.array_equal(runs[0], runs[1])


@pytest.mark.parametrize("n", [129, 192, 257, 1000, 1500])
def test_mixed_solve_stepped_triangular_solves(cuda, oracle, krr_system, n):
    # with cooperative launches off (batched and graph-recorded solves), the
    # triangular solves run one launch per pair of 64-row blocks (odd and even block
    # counts, full and short last blocks); the refined answer is the same
    X, y = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:n], X[:n], 1000.0))
    xr = oracle.refined_solve(K, y[:n], 1e-8)
    lib = core.lib()
    lib.qmlg_set_thread_cooperative(0)
    try:
        x, rep = core.solve(torch.from_numpy(K).to(cuda), torch.from_numpy(y[:n]).to(cuda), 1e-8,
                            precision="mixed")
    finally:
        lib.qmlg_set_thread_cooperative(1)
    assert rep["status"] == 0 and rep["fell_back"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-8, rep


def test_residual_dd_exact(cuda):
    rng = np.random.default_rng(0)
    A = rng.integers(-1000, 1000, size=(130, 130)).astype(np.float64)
    A = A + A.T
    x = rng.integers(-1000, 1000, size=130).astype(np.float64)
    y = A @ x + 3.0 * x
    At = torch.from_numpy(A).to(cuda)
    r = core.residual_dd(At, torch.from_numpy(np.diag(A).copy()).to(cuda), 3.0,
                         torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda))
    assert np.array_equal(r.cpu().numpy(), np.zeros(130))


def test_residual_is_correctly_rounded(cuda):
    # y - (A + lam I) x summed exactly (256-bit fixed point) and rounded once: every
    # row equals the correctly rounded exact value (Fractions), also under heavy
    # cancellation and with entries spread over many binades
    from fractions import Fraction
    rng = np.random.default_rng(7)
    n = 90
    A = rng.standard_normal((n, n)) * np.exp2(rng.integers(-30, 30, size=(n, n)))
    A = (A + A.T) / 2
    x = rng.standard_normal(n) * np.exp2(rng.integers(-20, 20, size=n))
    lam = 1e-3
    y = (A + lam * np.eye(n)) @ x * (1 + 1e-13 * rng.standard_normal(n))
    At = torch.from_numpy(A).to(cuda)
    r = core.residual_dd(At, torch.from_numpy(np.diag(A).copy()).to(cuda), lam,
                         torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)).cpu().numpy()
    for i in range(n):
        ex = Fraction(y[i]) - Fraction(lam) * Fraction(x[i]) - sum(
            Fraction(A[i, j]) * Fraction(x[j]) for j in range(n))
        assert r[i] == float(ex), (i, r[i], float(ex))


def _two_prod(a, b):
    """a * b = p + e exactly (Dekker's product with Veltkamp's split; no overflow or
    underflow in the ranges used here)."""
    def split(v):
        c = 134217729.0 * v
        hi = c - (c - v)
        return hi, v - hi
    p = a * b
    ah, al = split(a)
    bh, bl = split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


@pytest.mark.parametrize("n", [1100, 2100])
def test_residual_correctly_rounded_across_chunks(cuda, n):
    # several 1024-column chunks and 64-row blocks: mixed signs (so the sign of the
    # products differs across a warp), zeros, entries spread over 2^-250 .. 2^40 (so
    # products land above the head and far below the frame), and heavy cancellation.
    # Every row must equal the correctly rounded exact value: math.fsum of the exact
    # two-product pieces
    import math
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) * np.exp2(rng.integers(-40, 40, size=(n, n)))
    far = rng.random((n, n)) < 0.05
    A[far] *= 2.0 ** -200
    A[rng.random((n, n)) < 0.02] = 0.0
    A = np.triu(A) + np.triu(A, 1).T
    x = rng.standard_normal(n) * np.exp2(rng.integers(-20, 20, size=n))
    lam = 3e-7
    y = (A + lam * np.eye(n)) @ x * (1 + 1e-14 * rng.standard_normal(n))
    At = torch.from_numpy(A).to(cuda)
    r = core.residual_dd(At, torch.from_numpy(np.diag(A).copy()).to(cuda), lam,
                         torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)).cpu().numpy()
    p, e = _two_prod(A, x[None, :])
    lp, le = _two_prod(np.full(n, lam), x)
    ref = np.array([math.fsum(np.concatenate(([y[i], -lp[i], -le[i]], -p[i], -e[i])))
                    for i in range(n)])
    bad = np.nonzero(r != ref)[0]
    assert bad.size == 0, (bad[:5], r[bad[:5]], ref[bad[:5]])


@pytest.mark.parametrize("n", [65, 700, 1100, 1500])
def test_mixed_factor_matches_fp64_factor(cuda, oracle, krr_system, n):
    # the tensor-core factor (emulated FP64 trailing updates) against the plain FP64 one
    X, _ = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:n], X[:n], 500.0))
    lam = 1e-4
    Fm = torch.from_numpy(K).to(cuda)
    Fd = torch.from_numpy(K).to(cuda)
    assert core.cholesky(Fm, lam, precision="mixed") == 0
    assert core.cholesky(Fd, lam, precision="fp64") == 0
    Lm = np.tril(Fm.cpu().numpy())
    Ld = np.tril(Fd.cpu().numpy())
    assert np.max(np.abs(Lm - Ld)) <= 1e-11 * np.max(np.abs(Ld))
    # the other triangle is never written
    assert np.array_equal(np.triu(Fm.cpu().numpy(), 1), np.triu(K, 1))


def test_mixed_factor_info(cuda):
    from scipy.linalg import lapack
    rng = np.random.default_rng(2)
    M = rng.normal(size=(700, 700))
    S = M @ M.T + np.eye(700)
    S[600, 600] = -5.0
    _, info = lapack.dpotrf(np.asfortranarray(S), lower=0)
    St = torch.from_numpy(np.ascontiguousarray(S.T)).to(cuda)
    assert core.cholesky(St, precision="mixed") == info


def test_syrk_emulated(cuda):
    rng = np.random.default_rng(9)
    n, k = 300, 200
    P = rng.normal(size=(n, k)) * np.exp(rng.normal(size=(n, 1)))
    C = rng.normal(size=(n, n))
    Ct = torch.from_numpy(C).to(cuda)
    core.syrk_emulated(Ct, torch.from_numpy(P).to(cuda))
    out = Ct.cpu().numpy()
    ref = C - P @ P.T
    tri = np.tril_indices(n)
    scale = np.abs(P) @ np.abs(P).T + np.abs(C)
    assert np.max(np.abs(out[tri] - ref[tri]) / scale[tri]) < 1e-14
    assert np.array_equal(np.triu(out, 1), np.triu(C, 1))


def test_bounded_wait_gives_up(cuda, oracle, krr_system):
    # a wait on solved entries that nothing writes runs out after its poll limit and
    # the call reports QMLG_E_TIMEOUT; the context stays usable afterwards
    lib = core.lib()
    ws = torch.empty(lib.qmlg_selftest_wait_timeout_workspace_size(), dtype=torch.uint8,
                     device=cuda)
    st = lib.qmlg_selftest_wait_timeout(ws.data_ptr(), ws.numel(),
                                        torch.cuda.current_stream(cuda).cuda_stream)
    assert st == -6
    X, y = krr_system
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:300], X[:300], 1000.0))
    x, rep = core.solve(torch.from_numpy(K).to(cuda), torch.from_numpy(y[:300]).to(cuda), 1e-6,
                        precision="mixed")
    assert rep["status"] == 0, rep
    assert rel(x.cpu().numpy(), oracle.refined_solve(K, y[:300], 1e-6)) <= 1e-8


def test_mixed_solve_many_panels(cuda, oracle):
    # eight 512-column panels with the look-ahead between them, on an ill-conditioned
    # Gaussian K (lambda = 1e-8): alpha within 1e-8 of the refined oracle solve
    b = generate_molecules(4096, seed=77)
    X = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    K = np.ascontiguousarray(oracle.gaussian_kernel(X, X, 1000.0))
    xr = oracle.refined_solve(K, b.labels, 1e-8)
    x, rep = core.solve(torch.from_numpy(K).to(cuda), torch.from_numpy(b.labels).to(cuda), 1e-8,
                        precision="mixed")
    assert rep["status"] == 0 and rep["fell_back"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-8, rep


def test_mixed_fallback_refactorises_in_fp64(cuda, oracle, krr_system):
    # With four digit planes the tensor-core factor carries an error near 2^-28,
    # far too coarse for cond(K + 1e-8 I) ~ 1e10: refinement stalls (or a pivot
    # fails) and the solve restores the factorised triangle from the untouched one
    # and refactorises in FP64.  (fcho_solve.f90:36-42 prints a warning and carries
    # on after a failed dpotrf; here the FP64 factor takes over.)  The FP64
    # refinement then meets the same bar against the refined oracle.
    X, y = krr_system
    n, lam = 1500, 1e-8
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:n], X[:n], 1000.0))
    xr = oracle.refined_solve(K, y[:n], lam)
    A = torch.from_numpy(K).to(cuda)
    x, rep = core.solve(A, torch.from_numpy(y[:n]).to(cuda), lam, precision="mixed", slices=4)
    assert rep["fell_back"] == 1 and rep["precision_used"] == 0, rep
    assert rep["info"] == 0 and rep["status"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-8, rep
    F = A.cpu().numpy()
    # the other triangle (row-major strictly upper = column-major strictly lower) is K
    assert np.array_equal(np.triu(F, 1), np.triu(K, 1))
    # the factorised triangle holds an FP64 factor of K + lam I: U^T U = K + lam I to
    # FP64 backward-error level (the restore fed the FP64 factor the original K)
    L = np.tril(F)
    berr = np.linalg.norm(L @ L.T - (K + lam * np.eye(n))) / np.linalg.norm(K)
    assert berr <= 1e-14, berr


def test_mixed_fewer_planes_recover_when_well_conditioned(cuda, oracle, krr_system):
    # six planes at lambda = 1e-4 (cond ~ 1e7): refinement recovers, no fallback
    X, y = krr_system
    n, lam = 1500, 1e-4
    K = np.ascontiguousarray(oracle.gaussian_kernel(X[:n], X[:n], 1000.0))
    xr = oracle.refined_solve(K, y[:n], lam)
    x, rep = core.solve(torch.from_numpy(K).to(cuda), torch.from_numpy(y[:n]).to(cuda), lam,
                        precision="mixed", slices=6)
    assert rep["fell_back"] == 0 and rep["precision_used"] == 1 and rep["status"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-8, rep


def test_mixed_solve_not_positive_definite_falls_back_to_lapack_info(cuda):
    from scipy.linalg import lapack
    rng = np.random.default_rng(2)
    M = rng.normal(size=(700, 700))
    S = M @ M.T + np.eye(700)
    S[600, 600] = -5.0
    _, info = lapack.dpotrf(np.asfortranarray(S), lower=0)
    assert info > 0
    x, rep = core.solve(torch.from_numpy(S).to(cuda), torch.ones(700, dtype=torch.float64,
                        device=cuda), 0.0, precision="mixed", raise_on_info=False)
    assert rep["status"] == info and rep["info"] == info and rep["fell_back"] == 1, rep
    assert torch.isnan(x).all()


def test_solve_rejects_bad_plane_count(cuda):
    from qml_gb300._lib import QmlgError
    K = torch.eye(8, dtype=torch.float64, device=cuda)
    with pytest.raises(QmlgError):
        core.solve(K, torch.ones(8, dtype=torch.float64, device=cuda), 0.0, precision="mixed",
                   slices=3)
