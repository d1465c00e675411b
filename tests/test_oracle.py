"""The oracle (CPU restatement) against the reference's own known answers."""
import os

import numpy as np
import pytest

from conftest import load_golden, more_kernel_inputs
from qml_gb300.synthetic import generate_molecules

# The reference's source tree (read-only; its QM7 files feed the end-to-end check
# below, which is skipped where the tree is not mounted).
REF = os.environ.get("QML_REFERENCE_TREE", "/root/reference")


def test_cm_oracle_matches_reference_fixture(oracle):
    # tests/test_representations.py:46-90 (np.allclose against the text fixtures)
    g = load_golden("cm_qm7_0101_0110.npz")
    size = int(g["size"])
    off = g["offsets"]
    for m in range(off.shape[0] - 1):
        z = g["charges"][off[m]:off[m + 1]]
        r = g["coordinates"][off[m]:off[m + 1]]
        s = oracle.cm_sorted(z, r, size)
        u = oracle.cm_unsorted(z, r, size)
        assert np.allclose(s, g["sorted"][m]) and np.max(np.abs(s - g["sorted"][m])) < 1e-8
        assert np.allclose(u, g["unsorted"][m]) and np.max(np.abs(u - g["unsorted"][m])) < 1e-8
        assert np.array_equal(s, oracle.cm_sorted_numpy(z, r, size))


def test_cm_oracle_c_equals_numpy_restatement(oracle):
    b = generate_molecules(300, seed=11)
    X = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    for m in range(b.n_mol):
        z, r = b.molecule(m)
        assert np.array_equal(X[m], oracle.cm_sorted_numpy(z, r, 23))


def test_cm_tie_rule(oracle):
    # two hydrogens placed symmetrically about a carbon: equal row norms.  The
    # reference's repeated minloc places the lower index last, i.e. ties are ordered
    # by descending input index.
    z = np.array([1.0, 6.0, 1.0])
    r = np.array([[-1.1, 0.0, 0.0], [0.0, 0.0, 0.0], [1.1, 0.0, 0.0]])
    cm = oracle.cm_sorted(z, r, 3)
    full = np.zeros((3, 3))
    full[0, 0] = 0.5 * 6 ** 2.4
    # order should be C (1), then H index 2, then H index 0 -> M[2][0] = 1*1/2.2
    assert cm[0] == 0.5 * 6.0 ** 2.4
    assert cm[5] == 0.5 * 1.0 ** 2.4
    assert cm[4] == (1.0 * 1.0) / np.sqrt(2.2 * 2.2)
    assert np.array_equal(cm, oracle.cm_sorted_numpy(z, r, 3))


def test_cm_too_many_atoms(oracle):
    with pytest.raises(ValueError):
        oracle.cm_sorted(np.ones(5), np.zeros((5, 3)), 4)


def test_kernel_oracle_matches_reference_test(oracle):
    # tests/test_kernels.py:34-90
    g = load_golden("kernels_seed666.npz")
    K = oracle.laplacian_kernel(g["X"], g["Xs"], float(g["sigma"]))
    assert np.allclose(K, g["laplacian"])
    assert np.max(np.abs(K / g["laplacian"] - 1)) < 1e-12
    K = oracle.gaussian_kernel(g["X"], g["Xs"], float(g["sigma"]))
    assert np.allclose(K, g["gaussian"])
    assert np.max(np.abs(K / g["gaussian"] - 1)) < 1e-12
    Ks = oracle.gaussian_kernel(g["X"], g["X"], float(g["sigma"]))
    assert np.allclose(Ks, Ks.T)
    assert K.flags.f_contiguous


def _close(K, expect):
    # the reference test's bar (allclose) and this build's (1e-12 relative)
    return np.allclose(K, expect) and float(np.max(np.abs(K / expect - 1))) < 1e-12


def test_more_kernel_oracles_match_reference_tests(oracle):
    # tests/test_kernels.py:93-214: linear, Matern (L1 through the Sargan mapping of
    # qml/kernels.py:187-200, L2) and Sargan, on the same seeded inputs
    g = load_golden("kernels_more_seed666.npz")
    inp = more_kernel_inputs()
    s = float(g["sigma"])
    X, Xs = inp["linear"]
    K = oracle.linear_kernel(X, Xs)
    assert K.flags.f_contiguous and _close(K, g["linear"])
    l1_map = {0: ([], 1.0), 1: ([1.0], np.sqrt(3)), 2: ([1.0, 1 / 3.0], np.sqrt(5))}
    for order in (0, 1, 2):
        X, Xs = inp["matern_l2_%d" % order]
        assert _close(oracle.matern_kernel_l2(X, Xs, s, order), g["matern_l2_%d" % order])
        X, Xs = inp["matern_l1_%d" % order]
        gam, div = l1_map[order]
        assert _close(oracle.sargan_kernel(X, Xs, s / div, gam), g["matern_l1_%d" % order])
    for ng in (0, 1, 2):
        X, Xs = inp["sargan_%d" % ng]
        gam = inp["sargan_%d_gammas" % ng]
        assert np.array_equal(gam, g["sargan_%d_gammas" % ng])
        assert _close(oracle.sargan_kernel(X, Xs, s, gam), g["sargan_%d" % ng])
    # the Fortran's third Matern branch takes every other order
    X, Xs = inp["matern_l2_2"]
    assert np.array_equal(oracle.matern_kernel_l2(X, Xs, s, 5), oracle.matern_kernel_l2(X, Xs, s, 2))


ATOMIC_CUTOFFS = dict(central_cutoff=4.0, central_decay=0.5, interaction_cutoff=5.0,
                      interaction_decay=1.0)


def atomic_rows(oracle, g, sorting, central=None, **kw):
    z, r, off, size = g["charges"], g["coordinates"], g["offsets"], int(g["size"])
    return np.concatenate([oracle.atomic_cm(z[off[m]:off[m + 1]], r[off[m]:off[m + 1]], central,
                                            size, sorting, **kw) for m in range(len(off) - 1)])


def test_atomic_cm_oracle_matches_reference_fixtures(oracle):
    # tests/test_representations.py:92-158 on qm7/0101..0110 (size 17)
    g = load_golden("cm_qm7_0101_0110.npz")
    a = load_golden("atomic_cm_qm7_0101_0110.npz")
    for name, sorting, kw in (("distance_sorted", "distance", {}),
                              ("distance_sorted_no_indices", "distance", {}),
                              ("row-norm_sorted", "row-norm", {}),
                              ("distance_sorted_with_cutoff", "distance", ATOMIC_CUTOFFS),
                              ("row-norm_sorted_with_cutoff", "row-norm", ATOMIC_CUTOFFS)):
        X = atomic_rows(oracle, g, sorting, **kw)
        assert X.shape == a[name].shape and np.allclose(X, a[name]), name
    # central-atom subsets are the matching rows of the full set
    z, r, off = g["charges"], g["coordinates"], g["offsets"]
    for sorting in ("distance", "row-norm"):
        for m in range(10):
            zm, rm = z[off[m]:off[m + 1]], r[off[m]:off[m + 1]]
            full = oracle.atomic_cm(zm, rm, None, 17, sorting)
            assert np.array_equal(oracle.atomic_cm(zm, rm, [1, 2], 17, sorting), full[1:3])


def local_krr_features(oracle, L, sorting="row-norm"):
    z, r, off = L["charges"], L["coordinates"], L["offsets"]
    X = [oracle.atomic_cm(z[off[m]:off[m + 1]], r[off[m]:off[m + 1]], None, 23, sorting)
         for m in range(len(off) - 1)]
    n = np.array([x.shape[0] for x in X])
    return np.concatenate(X[:200]), np.concatenate(X[200:]), n[:200], n[200:]


def test_local_kernel_oracle_matches_reference_krr(oracle):
    # tests/test_energy_krr_atomic_cmat.py: K vs K_local_*.txt (allclose), Ks vs
    # Ks_local_*.txt (fewer than 5 molecules off by > 1e-7, the reference's
    # allowance), and the KRR mean absolute errors
    L = load_golden("local_krr_qm7.npz")
    X, Xs, N, Ns = local_krr_features(oracle, L)
    Y, Ys = L["energies"][:200], L["energies"][200:]
    for kind, sigma, lam, mae_ref in (("gaussian", 724.0, 10 ** (-6.5), 19.0),
                                      ("laplacian", 10 ** 3.6, 10 ** (-12.0), 8.7)):
        K = oracle.local_kernels(kind, X, X, N, N, [sigma])[0]
        assert np.allclose(K, K.T) and np.allclose(K, L["K_" + kind])
        Ks = oracle.local_kernels(kind, Xs, X, Ns, N, [sigma])[0]
        assert len(set(np.where(Ks - L["Ks_" + kind] > 1e-7)[0])) < 5
        K[np.diag_indices_from(K)] += lam
        alpha = oracle.cho_solve(K, Y)
        mae = np.mean(np.abs(Ys - Ks @ alpha))
        assert abs(mae_ref - mae) < 1.0, (kind, mae)


def test_cho_solve_oracle_matches_reference_test(oracle):
    # tests/test_math.py:32-52
    g = load_golden("cho_solve_k_local_gaussian.npz")
    x = oracle.cho_solve(g["A"], g["y"])
    assert np.allclose(x, np.linalg.solve(g["A"], g["y"]))


def test_cho_invert_oracle_matches_reference_test(oracle):
    # tests/test_math.py:54-71
    A = load_golden("cho_solve_k_local_gaussian.npz")["A"]
    Ai = oracle.cho_invert(A)
    assert np.allclose(A @ Ai, np.eye(A.shape[0]), atol=1e-7)
    assert np.array_equal(Ai, Ai.T)


def test_bkf_oracle_matches_reference_tests(oracle):
    # tests/test_math.py:74-112
    g = load_golden("cho_solve_k_local_gaussian.npz")
    A, y = g["A"], g["y"]
    x, info = oracle.bkf_solve(A, y)
    assert info == 0 and np.allclose(x, np.linalg.solve(A, y))
    Ai, info = oracle.bkf_invert(A)
    assert info == 0 and np.allclose(A @ Ai, np.eye(A.shape[0]), atol=1e-7)


def test_refined_solve_residual(oracle):
    b = generate_molecules(400, seed=5)
    X = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    K = np.ascontiguousarray(oracle.gaussian_kernel(X, X, 1000.0))
    for lam in (1e-4, 1e-8):
        x = oracle.refined_solve(K, b.labels, lam)
        r = oracle.residual_dd(K, lam, x, b.labels)
        # the refined residual sits at the rounding level of x itself
        assert np.linalg.norm(r) <= 1e-14 * np.linalg.norm(K, 1) * np.linalg.norm(x)
        x64 = oracle.cho_solve(K + lam * np.eye(K.shape[0]), b.labels)
        assert np.linalg.norm(x64 - x) / np.linalg.norm(x) < 1e-3


def test_residual_dd_exact_on_integers(oracle):
    rng = np.random.default_rng(0)
    A = rng.integers(-1000, 1000, size=(50, 50)).astype(np.float64)
    A = A + A.T
    x = rng.integers(-1000, 1000, size=50).astype(np.float64)
    y = A @ x + 3.0 * x
    assert np.array_equal(oracle.residual_dd(A, 3.0, x, y), np.zeros(50))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "tests", "qm7")),
                    reason="reference tree not mounted")
def test_oracle_krr_cmat_reference_accuracy(oracle):
    # tests/test_energy_krr_cmat.py:54-113 run on the oracle: MAE < 6.0
    from qml_gb300.compound import Compound
    energies = {}
    with open(os.path.join(REF, "tests/data/hof_qm7.txt")) as f:
        for line in f:
            t = line.split()
            energies[t[0]] = float(t[1])
    mols = []
    for name in sorted(energies.keys())[:1000]:
        c = Compound(os.path.join(REF, "tests/qm7", name))
        c.properties = energies[name]
        mols.append(c)
    np.random.seed(666)
    np.random.shuffle(mols)
    train, test = mols[:700], mols[-300:]
    X = np.array([oracle.cm_sorted(m.nuclear_charges, m.coordinates, 23) for m in train])
    Xs = np.array([oracle.cm_sorted(m.nuclear_charges, m.coordinates, 23) for m in test])
    Y = np.array([m.properties for m in train])
    Ys = np.array([m.properties for m in test])
    sigma = 10 ** 4.2
    K = oracle.laplacian_kernel(X, X, sigma)
    K[np.diag_indices_from(K)] += 1e-10
    alpha = oracle.cho_solve(K, Y)
    Ks = oracle.laplacian_kernel(X, Xs, sigma)
    mae = np.mean(np.abs(Ys - Ks.T @ alpha))
    assert mae < 6.0


def test_rows_residual_dd_matches_square_residual(oracle):
    # the rectangular double-double residual equals the square one on the same rows
    rng = np.random.default_rng(4)
    A = rng.normal(size=(60, 60))
    A = A + A.T
    x = rng.normal(size=60)
    y = rng.normal(size=60)
    full = oracle.residual_dd(A, 0.0, x, y)
    rows = np.array([0, 7, 33, 59])
    part = oracle.rows_residual_dd(A[rows], x, y[rows])
    assert np.array_equal(part, full[rows])
