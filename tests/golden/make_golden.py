"""Builds the golden fixtures in this folder from the reference's own test data.

Run where the reference tree is mounted: pass its path, or set QML_REFERENCE_TREE
(default /root/reference).  Without the tree the script exits with a message.
Outputs (small .npz files, committed):
  cm_qm7_0101_0110.npz  inputs and expected outputs of the reference's Coulomb-matrix
                        known-answer test (tests/test_representations.py:46-90):
                        Z, R of qm7/0101..0110.xyz, size = max natoms + 1 = 17,
                        row-norm sorted and unsorted vectors (10 x 153) from
                        tests/data/coulomb_matrix_representation_*.txt
  cho_solve_k_local_gaussian.npz
                        the SPD system of tests/test_math.py:32-52:
                        A = tests/data/K_local_gaussian.txt (200 x 200),
                        y = tests/data/y_cho_solve.txt (200)
  kernels_seed666.npz   the inputs of tests/test_kernels.py:34-90 (np.random.seed(666),
                        X = rand(25, 1000), Xs = rand(20, 1000), sigma = 100) with the
                        reference test's own NumPy-loop expectations
  atomic_cm_qm7_0101_0110.npz
                        the reference's atomic Coulomb-matrix known answers
                        (tests/test_representations.py:92-158) for the same ten
                        molecules: distance- and row-norm-sorted, with and without the
                        soft cutoffs (central 4.0/0.5, interaction 5.0/1.0), from
                        tests/data/atomic_coulomb_matrix_representation_*.txt
  local_krr_qm7.npz     the atomic-CM KRR tests (tests/test_energy_krr_atomic_cmat.py):
                        the 200 training and 100 test molecules that the test's seed-666
                        shuffle of the first 1000 sorted QM7 names selects (Z, R, heats
                        of formation) and tests/data/K_local_*.txt, Ks_local_*.txt
  kernels_more_seed666.npz
                        the NumPy-loop expectations of tests/test_kernels.py:93-214
                        (linear, Matern and Sargan kernels) and the Sargan gammas; the
                        inputs are not stored: tests redraw them with
                        more_kernel_inputs() (NumPy's legacy seeded stream is frozen)
"""
import os
import sys

import numpy as np

NC = {"H": 1, "C": 6, "N": 7, "O": 8, "S": 16}


def read_xyz(path):
    with open(path) as f:
        lines = f.readlines()
    n = int(lines[0])
    z, r = [], []
    for line in lines[2:2 + n]:
        t = line.split()
        z.append(NC[t[0]])
        r.append([float(v) for v in t[1:4]])
    return np.array(z, dtype=np.float64), np.array(r, dtype=np.float64)


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    mols = [read_xyz(os.path.join(ref, "tests", "qm7", "%04d.xyz" % k)) for k in range(101, 111)]
    size = max(z.shape[0] for z, _ in mols) + 1
    counts = np.array([z.shape[0] for z, _ in mols], dtype=np.int64)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    np.savez_compressed(
        os.path.join(here, "cm_qm7_0101_0110.npz"),
        charges=np.concatenate([z for z, _ in mols]),
        coordinates=np.concatenate([r for _, r in mols]),
        offsets=offsets, size=size,
        sorted=np.loadtxt(os.path.join(ref, "tests/data/coulomb_matrix_representation_row-norm_sorted.txt")),
        unsorted=np.loadtxt(os.path.join(ref, "tests/data/coulomb_matrix_representation_unsorted.txt")))
    np.savez_compressed(
        os.path.join(here, "cho_solve_k_local_gaussian.npz"),
        A=np.loadtxt(os.path.join(ref, "tests/data/K_local_gaussian.txt")),
        y=np.loadtxt(os.path.join(ref, "tests/data/y_cho_solve.txt")))
    np.random.seed(666)
    X = np.random.rand(25, 1000)
    Xs = np.random.rand(20, 1000)
    sigma = 100.0
    kl = np.zeros((25, 20))
    kg = np.zeros((25, 20))
    for i in range(25):
        for j in range(20):
            kl[i, j] = np.exp(np.sum(np.abs(X[i] - Xs[j])) / (-1.0 * sigma))
            kg[i, j] = np.exp(np.sum(np.square(X[i] - Xs[j])) / (-2.0 * sigma ** 2))
    np.savez_compressed(os.path.join(here, "kernels_seed666.npz"), X=X, Xs=Xs, sigma=sigma,
                        laplacian=kl, gaussian=kg)
    more_kernels(here)
    atomic(ref, here)
    local_krr(ref, here)


def atomic(ref, here):
    d = os.path.join(ref, "tests", "data")
    names = ["distance_sorted", "distance_sorted_no_indices", "row-norm_sorted",
             "distance_sorted_with_cutoff", "row-norm_sorted_with_cutoff"]
    np.savez_compressed(os.path.join(here, "atomic_cm_qm7_0101_0110.npz"),
                        **{n: np.loadtxt(os.path.join(d, "atomic_coulomb_matrix_representation_%s.txt" % n))
                           for n in names})


def local_krr(ref, here):
    energies = {}
    with open(os.path.join(ref, "tests", "data", "hof_qm7.txt")) as f:
        for line in f:
            t = line.split()
            energies[t[0]] = float(t[1])
    names = sorted(energies.keys())[:1000]
    idx = list(range(len(names)))
    np.random.seed(666)
    np.random.shuffle(idx)
    sel = idx[:200] + idx[-100:]
    mols = [read_xyz(os.path.join(ref, "tests", "qm7", names[k])) for k in sel]
    counts = np.array([z.shape[0] for z, _ in mols], dtype=np.int64)
    d = os.path.join(ref, "tests", "data")
    np.savez_compressed(
        os.path.join(here, "local_krr_qm7.npz"),
        charges=np.concatenate([z for z, _ in mols]),
        coordinates=np.concatenate([r for _, r in mols]),
        offsets=np.concatenate([[0], np.cumsum(counts)]).astype(np.int64),
        energies=np.array([energies[names[k]] for k in sel]),
        K_gaussian=np.loadtxt(os.path.join(d, "K_local_gaussian.txt")),
        Ks_gaussian=np.loadtxt(os.path.join(d, "Ks_local_gaussian.txt")),
        K_laplacian=np.loadtxt(os.path.join(d, "K_local_laplacian.txt")),
        Ks_laplacian=np.loadtxt(os.path.join(d, "Ks_local_laplacian.txt")))


def more_kernel_inputs():
    """The inputs of tests/test_kernels.py:93-214, in draw order: each of those tests
    seeds 666 once and draws its inputs in sequence (Matern: l1 then l2, orders 0, 1,
    2; Sargan: 0, 1, 2 gammas, each followed by X and Xs).  Returns a dict of
    key -> (X, Xs) and key -> gammas for the Sargan cases."""
    out = {}
    np.random.seed(666)
    out["linear"] = (np.random.rand(25, 1000), np.random.rand(20, 1000))
    np.random.seed(666)
    for metric in ("l1", "l2"):
        for order in (0, 1, 2):
            out["matern_%s_%d" % (metric, order)] = (np.random.rand(25, 1000),
                                                    np.random.rand(20, 1000))
    np.random.seed(666)
    for ng in (0, 1, 2):
        gammas = np.random.random(ng)
        out["sargan_%d" % ng] = (np.random.rand(25, 1000), np.random.rand(20, 1000))
        out["sargan_%d_gammas" % ng] = gammas
    return out


def more_kernels(here):
    """Expectations of tests/test_kernels.py:93-214, computed by those tests' loops."""
    inp = more_kernel_inputs()
    sigma = 100.0
    out = {"sigma": sigma}
    X, Xs = inp["linear"]
    out["linear"] = np.array([[np.dot(X[i], Xs[j]) for j in range(20)] for i in range(25)])
    for metric in ("l1", "l2"):
        for order in (0, 1, 2):
            X, Xs = inp["matern_%s_%d" % (metric, order)]
            K = np.zeros((25, 20))
            for i in range(25):
                for j in range(20):
                    if metric == "l1":
                        d = np.sum(abs(X[i] - Xs[j]))
                    else:
                        d = np.sqrt(np.sum((X[i] - Xs[j]) ** 2))
                    if order == 0:
                        K[i, j] = np.exp(-d / sigma)
                    elif order == 1:
                        K[i, j] = np.exp(-np.sqrt(3) * d / sigma) * (1 + np.sqrt(3) * d / sigma)
                    else:
                        K[i, j] = np.exp(-np.sqrt(5) * d / sigma) * \
                            (1 + np.sqrt(5) * d / sigma + 5.0 / 3 * d ** 2 / sigma ** 2)
            out["matern_%s_%d" % (metric, order)] = K
    for ng in (0, 1, 2):
        gammas = inp["sargan_%d_gammas" % ng]
        X, Xs = inp["sargan_%d" % ng]
        K = np.zeros((25, 20))
        for i in range(25):
            for j in range(20):
                d = np.sum(abs(X[i] - Xs[j]))
                factor = 1
                for k, gamma in enumerate(gammas):
                    factor += gamma / sigma ** (k + 1) * d ** (k + 1)
                K[i, j] = np.exp(-d / sigma) * factor
        out["sargan_%d" % ng] = K
        out["sargan_%d_gammas" % ng] = gammas
    np.savez_compressed(os.path.join(here, "kernels_more_seed666.npz"), **out)


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QML_REFERENCE_TREE",
                                                                 "/root/reference")
    if not os.path.isdir(os.path.join(tree, "tests", "data")):
        sys.exit("reference tree not found at %s (pass its path or set QML_REFERENCE_TREE)" % tree)
    main(tree)
