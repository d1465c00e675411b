"""Atomic Coulomb matrices and local kernels on the GPU against the oracle and the
reference's fixtures (tests/test_representations.py:92-158,
tests/test_energy_krr_atomic_cmat.py)."""
import numpy as np
import pytest
import torch

from conftest import load_golden
from test_oracle import ATOMIC_CUTOFFS, atomic_rows, local_krr_features
from qml_gb300 import core
from qml_gb300.compound import Compound
from qml_gb300.kernels import get_local_kernels_gaussian, get_local_kernels_laplacian
from qml_gb300.math import cho_solve
from qml_gb300.representations import (generate_atomic_coulomb_matrix,
                                       generate_atomic_coulomb_matrix_batch)
from qml_gb300.synthetic import generate_molecules
from qml_gb300.wrappers import get_atomic_kernels_gaussian, get_atomic_kernels_laplacian

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def relerr(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def drop_in_rows(g, sorting, **kw):
    z, r, off, size = g["charges"], g["coordinates"], g["offsets"], int(g["size"])
    return np.concatenate([generate_atomic_coulomb_matrix(z[off[m]:off[m + 1]], r[off[m]:off[m + 1]],
                                                          size=size, sorting=sorting, **kw)
                           for m in range(len(off) - 1)])


def test_atomic_cm_reference_fixtures(cuda, oracle):
    # the reference's known answers through the drop-in; without cutoffs bit-identical
    # to the oracle's restatement, with the soft cutoffs (device cos) within 1e-13
    g = load_golden("cm_qm7_0101_0110.npz")
    a = load_golden("atomic_cm_qm7_0101_0110.npz")
    for name, sorting, kw in (("distance_sorted", "distance", {}),
                              ("row-norm_sorted", "row-norm", {}),
                              ("distance_sorted_with_cutoff", "distance", ATOMIC_CUTOFFS),
                              ("row-norm_sorted_with_cutoff", "row-norm", ATOMIC_CUTOFFS)):
        X = drop_in_rows(g, sorting, **kw)
        assert np.allclose(X, a[name]), name
        Xo = atomic_rows(oracle, g, sorting, **kw)
        if kw:
            assert np.max(np.abs(X - Xo)) <= 1e-13 * np.max(np.abs(Xo)), name
        else:
            assert np.array_equal(X, Xo), name


def test_atomic_cm_indices(cuda, oracle):
    g = load_golden("cm_qm7_0101_0110.npz")
    z, r, off = g["charges"], g["coordinates"], g["offsets"]
    for sorting in ("distance", "row-norm"):
        for m in range(10):
            zm, rm = z[off[m]:off[m + 1]], r[off[m]:off[m + 1]]
            full = generate_atomic_coulomb_matrix(zm, rm, size=17, sorting=sorting)
            sub = generate_atomic_coulomb_matrix(zm, rm, size=17, sorting=sorting, indices=[1, 2])
            assert np.array_equal(sub, full[1:3])
            carbons = generate_atomic_coulomb_matrix(zm, rm, size=17, sorting=sorting, indices="C")
            assert np.array_equal(carbons, full[zm == 6])
    zm, rm = z[off[0]:off[1]], r[off[0]:off[1]]
    assert generate_atomic_coulomb_matrix(zm, rm, size=17, indices="Cl").shape == (0, 0)
    with pytest.raises(SystemExit):
        generate_atomic_coulomb_matrix(zm, rm, size=17, indices="Xx")
    with pytest.raises(SystemExit):
        generate_atomic_coulomb_matrix(zm, rm, size=17, sorting="eigen")
    with pytest.raises(Exception):
        generate_atomic_coulomb_matrix(zm, rm, size=3)  # more atoms in the cutoff than size


@pytest.mark.parametrize("sorting", ["distance", "row-norm"])
def test_atomic_cm_batch_mixed_paths(cuda, oracle, sorting):
    # a cutoff that only some molecules reach: in one launch, the molecules it does
    # not touch take the one-pass path (bit-exact), the others the per-centre steps
    # (within 1e-13: the device cos); with central-atom subsets as well
    b = generate_molecules(400, seed=21)
    kw = dict(central_cutoff=6.0, central_decay=1.0, interaction_cutoff=9.0, interaction_decay=1.0)
    span = np.array([np.max(np.linalg.norm(r[:, None] - r[None], axis=-1))
                     for r in (b.molecule(m)[1] for m in range(400))])
    inside = span <= 5.0
    assert 20 < inside.sum() < 380
    X = generate_atomic_coulomb_matrix_batch(b.charges, b.coordinates, b.offsets, size=23,
                                             sorting=sorting, **kw).cpu().numpy()
    rows = [oracle.atomic_cm(*b.molecule(m), None, 23, sorting, **kw) for m in range(400)]
    Xo = np.concatenate(rows)
    start = np.concatenate([[0], np.cumsum([r.shape[0] for r in rows])])
    for m in range(400):
        got, want = X[start[m]:start[m + 1]], Xo[start[m]:start[m + 1]]
        if inside[m]:
            assert np.array_equal(got, want), m
        else:
            assert np.max(np.abs(got - want)) <= 1e-13 * max(1.0, np.max(np.abs(want))), m
    # every second atom as centre, through the C ABI's central subsets
    z, r, o = (torch.from_numpy(x).to(cuda) for x in (b.charges, b.coordinates, b.offsets))
    cen = [np.arange(0, b.offsets[m + 1] - b.offsets[m], 2) for m in range(400)]
    coff = torch.from_numpy(np.concatenate([[0], np.cumsum([c.shape[0] for c in cen])])).to(cuda)
    cat = torch.from_numpy(np.concatenate(cen).astype(np.int32)).to(cuda)
    Xs = core.atomic_coulomb_matrix_batch(z, r, o, 23, sorting, central_offsets=coff,
                                          central_atoms=cat, **kw).cpu().numpy()
    want = np.concatenate([oracle.atomic_cm(*b.molecule(m), cen[m], 23, sorting, **kw)
                           for m in range(400)])
    assert np.max(np.abs(Xs - want)) <= 1e-13 * np.max(np.abs(want))


@pytest.mark.parametrize("sorting", ["distance", "row-norm"])
def test_atomic_cm_batch_bit_exact(cuda, oracle, sorting):
    # one launch over a synthetic batch against the per-molecule oracle
    b = generate_molecules(300, seed=11)
    X = generate_atomic_coulomb_matrix_batch(b.charges, b.coordinates, b.offsets, size=23,
                                             sorting=sorting).cpu().numpy()
    Xo = np.concatenate([oracle.atomic_cm(*b.molecule(m), None, 23, sorting) for m in range(300)])
    assert np.array_equal(X, Xo)


def test_local_kernels_vs_oracle(cuda, oracle):
    L = load_golden("local_krr_qm7.npz")
    X, Xs, N, Ns = local_krr_features(oracle, L)
    sigmas = [200.0, 724.0, 10 ** 3.6]
    for kind, fn in (("gaussian", get_local_kernels_gaussian),
                     ("laplacian", get_local_kernels_laplacian)):
        K = fn(X, X, N, N, sigmas)
        assert K.shape == (3, 200, 200) and K.flags.f_contiguous
        assert relerr(K, oracle.local_kernels(kind, X, X, N, N, sigmas)) <= RTOL
        for s in range(3):
            assert np.array_equal(K[s], K[s].T)
        Ks = fn(Xs, X, Ns, N, sigmas)
        assert relerr(Ks, oracle.local_kernels(kind, Xs, X, Ns, N, sigmas)) <= RTOL


def test_local_krr_reference_end_to_end(cuda):
    # tests/test_energy_krr_atomic_cmat.py with every step on the GPU: atomic CMs
    # through Compound, local kernels, the reference's fixtures and KRR errors
    L = load_golden("local_krr_qm7.npz")
    z, r, off = L["charges"], L["coordinates"], L["offsets"]
    mols = []
    for m in range(300):
        c = Compound()
        c.nuclear_charges = z[off[m]:off[m + 1]].astype(int)
        c.coordinates = r[off[m]:off[m + 1]]
        c.natoms = int(off[m + 1] - off[m])
        c.generate_atomic_coulomb_matrix(size=23, sorting="row-norm")
        mols.append(c)
    training, test = mols[:200], mols[200:]
    X = np.concatenate([m.representation for m in training])
    Xs = np.concatenate([m.representation for m in test])
    N = np.array([m.natoms for m in training])
    Ns = np.array([m.natoms for m in test])
    Y, Ys = L["energies"][:200], L["energies"][200:]
    for kind, fn, wrap, sigma, lam, mae_ref in (
            ("gaussian", get_local_kernels_gaussian, get_atomic_kernels_gaussian, 724.0,
             10 ** (-6.5), 19.0),
            ("laplacian", get_local_kernels_laplacian, get_atomic_kernels_laplacian, 10 ** 3.6,
             10 ** (-12.0), 8.7)):
        K = fn(X, X, N, N, [sigma])[0]
        assert np.allclose(K, K.T) and np.allclose(K, L["K_" + kind])
        assert np.allclose(K, wrap(training, training, [sigma])[0])
        Ks = fn(Xs, X, Ns, N, [sigma])[0]
        assert len(set(np.where(Ks - L["Ks_" + kind] > 1e-7)[0])) < 5
        assert np.allclose(Ks, wrap(test, training, [sigma])[0])
        K = np.ascontiguousarray(K)
        K[np.diag_indices_from(K)] += lam
        alpha = cho_solve(K, Y)
        mae = np.mean(np.abs(Ys - Ks @ alpha))
        assert abs(mae_ref - mae) < 1.0, (kind, mae)


def test_local_kernels_emulated_vs_oracle(cuda, oracle):
    # atom-pair matrices from the tensor-core Gaussian / fixed-point Laplacian, summed
    # per molecule pair: within 1e-12 per entry, exactly symmetric in symmetric mode
    L = load_golden("local_krr_qm7.npz")
    X, Xs, N, Ns = local_krr_features(oracle, L)
    sigmas = [200.0, 724.0, 10 ** 3.6]
    Xt, Xst = torch.from_numpy(X).to(cuda), torch.from_numpy(Xs).to(cuda)
    off = torch.from_numpy(np.concatenate([[0], np.cumsum(N)])).to(cuda)
    offs = torch.from_numpy(np.concatenate([[0], np.cumsum(Ns)])).to(cuda)
    for kind in ("gaussian", "laplacian"):
        K = core.local_kernels(kind, Xt, Xt, off, off, sigmas, symmetric=True,
                               emulated=True).cpu().numpy()
        assert relerr(K, oracle.local_kernels(kind, X, X, N, N, sigmas)) <= RTOL
        for s in range(3):
            assert np.array_equal(K[s], K[s].T)
        Ks = core.local_kernels(kind, Xst, Xt, offs, off, sigmas, emulated=True).cpu().numpy()
        assert relerr(Ks, oracle.local_kernels(kind, Xs, X, Ns, N, sigmas)) <= RTOL


def test_local_kernels_emulated_chunks_and_empty_molecules(cuda):
    # 70000 B atoms hold a chunk to 4096 A rows, so 600 A molecules take three chunks;
    # molecules without atoms give zeros.  Held to the FP64 local kernel (itself
    # pinned to the oracle above)
    ba = generate_molecules(600, seed=11)
    bb = generate_molecules(5000, seed=12)
    za, ra, oa = (torch.from_numpy(x).to(cuda) for x in (ba.charges, ba.coordinates, ba.offsets))
    zb, rb, ob = (torch.from_numpy(x).to(cuda) for x in (bb.charges, bb.coordinates, bb.offsets))
    A = core.atomic_coulomb_matrix_batch(za, ra, oa, 23, "row-norm")
    B = core.atomic_coulomb_matrix_batch(zb, rb, ob, 23, "row-norm")
    assert A.shape[0] > 8192 and B.shape[0] > 65536
    for kind, sig in (("gaussian", [724.0]), ("laplacian", [10 ** 3.6])):
        Ke = core.local_kernels(kind, A, B, oa, ob, sig, emulated=True).cpu().numpy()
        Kf = core.local_kernels(kind, A, B, oa, ob, sig).cpu().numpy()
        assert relerr(Ke, Kf) <= RTOL
    # a symmetric problem past one chunk (about 21000 atoms, chunks of 2 GiB hold
    # 12800): each chunk starts at its own first atom, the mirror fills the rest
    bs = generate_molecules(1500, seed=13)
    zs, rs, os_ = (torch.from_numpy(x).to(cuda) for x in (bs.charges, bs.coordinates, bs.offsets))
    S = core.atomic_coulomb_matrix_batch(zs, rs, os_, 23, "row-norm")
    assert S.shape[0] > 2 ** 31 // (8 * S.shape[0])
    for kind, sig in (("gaussian", [724.0, 2000.0]), ("laplacian", [10 ** 3.6])):
        Ke = core.local_kernels(kind, S, S, os_, os_, sig, symmetric=True, emulated=True).cpu().numpy()
        Kf = core.local_kernels(kind, S, S, os_, os_, sig, symmetric=True).cpu().numpy()
        assert relerr(Ke, Kf) <= RTOL
        for k in range(len(sig)):
            assert np.array_equal(Ke[k], Ke[k].T)
    # empty molecules at the ends and in the middle
    n = np.array([0, 5, 0, 7, 3, 0])
    rows = torch.from_numpy(np.random.default_rng(5).uniform(0, 50, (int(n.sum()), 40))).to(cuda)
    o = torch.from_numpy(np.concatenate([[0], np.cumsum(n)])).to(cuda)
    Ke = core.local_kernels("gaussian", rows, rows, o, o, [30.0], symmetric=True,
                            emulated=True).cpu().numpy()
    Kf = core.local_kernels("gaussian", rows, rows, o, o, [30.0], symmetric=True).cpu().numpy()
    empty = n == 0
    assert np.all(Ke[0][empty, :] == 0) and np.all(Ke[0][:, empty] == 0)
    full = ~empty
    assert relerr(Ke[0][np.ix_(full, full)], Kf[0][np.ix_(full, full)]) <= RTOL
