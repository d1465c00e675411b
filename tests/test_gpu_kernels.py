"""Kernel matrices (Gaussian, Laplacian, linear, Matern, Sargan) and prediction on
the GPU vs the oracle (relative error <= 1e-12 per entry, the FP64-path bar)."""
import numpy as np
import pytest
import torch

from conftest import load_golden, more_kernel_inputs
from qml_gb300 import _lib, core
from qml_gb300.kernels import (gaussian_kernel, laplacian_kernel, linear_kernel, matern_kernel,
                               sargan_kernel)
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def relerr(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def test_reference_kernel_test(cuda, oracle):
    # tests/test_kernels.py:34-90 through the drop-in API
    g = load_golden("kernels_seed666.npz")
    X, Xs, s = g["X"], g["Xs"], float(g["sigma"])
    for fn, key, ofn in ((laplacian_kernel, "laplacian", oracle.laplacian_kernel),
                         (gaussian_kernel, "gaussian", oracle.gaussian_kernel)):
        K = fn(X, Xs, s)
        assert K.flags.f_contiguous and K.shape == (25, 20)
        assert np.allclose(K, g[key])
        assert relerr(K, ofn(X, Xs, s)) <= RTOL
        Ks = fn(X, X, s)
        assert np.array_equal(Ks, Ks.T)
        assert relerr(Ks, ofn(X, X, s)) <= RTOL


@pytest.fixture(scope="module")
def cm_features(oracle):
    b = generate_molecules(1000, seed=7)
    return oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)


@pytest.mark.parametrize("kind", ["gaussian", "laplacian"])
@pytest.mark.parametrize("sigma", [250.0, 1000.0, 2000.0])
def test_cm_features(cuda, oracle, cm_features, kind, sigma):
    X = cm_features
    A, B = X[:700], X[700:]
    ofn = oracle.gaussian_kernel if kind == "gaussian" else oracle.laplacian_kernel
    At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    K = core.kernel_matrix(kind, At, Bt, sigma).cpu().numpy()
    assert relerr(K, ofn(A, B, sigma)) <= RTOL
    Ks = core.kernel_matrix(kind, At, At, sigma, symmetric=True).cpu().numpy()
    assert np.array_equal(Ks, Ks.T)
    assert relerr(Ks, ofn(A, A, sigma)) <= RTOL


@pytest.mark.parametrize("na,nb,d", [(1, 1, 1), (1, 65, 17), (65, 1, 276), (130, 67, 33), (64, 64, 16)])
def test_odd_shapes(cuda, oracle, na, nb, d):
    rng = np.random.default_rng(na * 1000 + nb)
    A = rng.random((na, d)) * 10
    B = rng.random((nb, d)) * 10
    for kind, ofn in (("gaussian", oracle.gaussian_kernel), ("laplacian", oracle.laplacian_kernel)):
        K = core.kernel_matrix(kind, torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda),
                               7.0).cpu().numpy()
        assert relerr(K, ofn(A, B, 7.0)) <= RTOL


def test_diag_shift(cuda, cm_features):
    At = torch.from_numpy(cm_features[:100]).to(cuda)
    K0 = core.kernel_matrix("gaussian", At, At, 1000.0, symmetric=True)
    K1 = core.kernel_matrix("gaussian", At, At, 1000.0, symmetric=True, diag_shift=0.5)
    d = (K1 - K0).cpu().numpy()
    assert np.array_equal(np.diag(d), np.full(100, 0.5)) and np.count_nonzero(d) == 100


@pytest.mark.parametrize("kind", ["gaussian", "laplacian"])
def test_predict_fused_and_gemv(cuda, oracle, cm_features, kind):
    rng = np.random.default_rng(3)
    Xtr, Xte = cm_features[:900], cm_features[900:]
    alpha = rng.normal(size=900)
    ofn = oracle.gaussian_kernel if kind == "gaussian" else oracle.laplacian_kernel
    Ks = ofn(Xtr, Xte, 1000.0)
    expect = Ks.T @ alpha
    y = core.predict(kind, torch.from_numpy(Xtr).to(cuda), torch.from_numpy(Xte).to(cuda), 1000.0,
                     torch.from_numpy(alpha).to(cuda)).cpu().numpy()
    scale = np.abs(Ks.T) @ np.abs(alpha)
    assert np.max(np.abs(y - expect) / scale) <= 1e-12
    y2 = core.predict_gemv(torch.from_numpy(np.asfortranarray(Ks)).to(cuda).T.contiguous().T,
                           torch.from_numpy(alpha).to(cuda)).cpu().numpy()
    assert np.max(np.abs(y2 - expect) / scale) <= 1e-13
    # deterministic: bitwise identical on a second call
    y3 = core.predict(kind, torch.from_numpy(Xtr).to(cuda), torch.from_numpy(Xte).to(cuda), 1000.0,
                      torch.from_numpy(alpha).to(cuda)).cpu().numpy()
    assert np.array_equal(y, y3)


@pytest.mark.parametrize("sigma", [1000.0, 1e5])
def test_predict_laplacian_fixed(cuda, oracle, cm_features, sigma):
    # fused Laplacian prediction with fixed-point L1 sums (and the FP64 kernel when the
    # grid cannot meet the bound, sigma = 1e5 still fits): within 1e-12 of the oracle
    # relative to sum |k alpha|, deterministic
    rng = np.random.default_rng(5)
    Xtr, Xte = cm_features[:900], cm_features[900:]
    alpha = rng.normal(size=900)
    Ks = oracle.laplacian_kernel(Xtr, Xte, sigma)
    expect = Ks.T @ alpha
    scale = np.abs(Ks.T) @ np.abs(alpha)
    args = (torch.from_numpy(Xtr).to(cuda), torch.from_numpy(Xte).to(cuda), sigma,
            torch.from_numpy(alpha).to(cuda))
    y = core.predict("laplacian", *args, emulated=True).cpu().numpy()
    assert np.max(np.abs(y - expect) / scale) <= 1e-12
    assert np.array_equal(y, core.predict("laplacian", *args, emulated=True).cpu().numpy())


@pytest.mark.parametrize("sigma", [250.0, 1000.0, 2000.0])
def test_emulated_gaussian_kernel(cuda, oracle, cm_features, sigma):
    # tensor-core (digit-plane) contraction: every entry within 1e-12 of the oracle
    X = cm_features
    A, B = X[:700], X[700:]
    At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    K = core.kernel_matrix("gaussian", At, Bt, sigma, emulated=True).cpu().numpy()
    assert relerr(K, oracle.gaussian_kernel(A, B, sigma)) <= RTOL
    Ks = core.kernel_matrix("gaussian", At, At, sigma, symmetric=True, emulated=True,
                            diag_shift=0.25).cpu().numpy()
    assert np.array_equal(Ks, Ks.T)
    Ko = oracle.gaussian_kernel(A, A, sigma)
    Ko[np.diag_indices_from(Ko)] += 0.25
    assert relerr(Ks, Ko) <= RTOL


@pytest.mark.parametrize("na,nb", [(1, 1), (129, 65), (300, 1000)])
def test_emulated_gaussian_odd_shapes(cuda, oracle, cm_features, na, nb):
    A, B = cm_features[:na], cm_features[1000 - nb:]
    K = core.kernel_matrix("gaussian", torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda),
                           1000.0, emulated=True).cpu().numpy()
    assert relerr(K, oracle.gaussian_kernel(A, B, 1000.0)) <= RTOL


def test_emulated_gaussian_small_sigma_falls_back(cuda, oracle):
    g = load_golden("kernels_seed666.npz")
    X, Xs = g["X"], g["Xs"]
    for s in (0.05, 100.0):
        K = core.kernel_matrix("gaussian", torch.from_numpy(X).to(cuda), torch.from_numpy(Xs).to(cuda),
                               s, emulated=True).cpu().numpy()
        Ko = oracle.gaussian_kernel(X, Xs, s)
        assert np.allclose(K, Ko, rtol=1e-12, atol=0)


@pytest.mark.parametrize("lo,hi", [(-700.0, 0.0), (-1.0, 0.0), (-1e-3, 0.0), (-5.0, -4.0),
                                   (-700.0, -600.0), (-1e-12, 0.0)])
def test_epilogue_exp_against_library_exp(cuda, lo, hi):
    # the fixed-point exp of the Gaussian epilogues: within 2 ulp of the host libm and
    # of CUDA's exp (torch.exp) over a million arguments per range
    rng = np.random.default_rng(int(-lo * 1000) + 7)
    x = rng.uniform(lo, hi, 1 << 20)
    x[:8] = [lo, hi, -0.0, 0.0, -1e-300, -np.log(2.0), -1.0, -699.9999]
    xt = torch.from_numpy(x).to(cuda)
    y = torch.empty_like(xt)
    assert core.lib().qmlg_epilogue_exp(xt.data_ptr(), y.data_ptr(), x.size,
                                        torch.cuda.current_stream().cuda_stream) == 0
    y = y.cpu().numpy()
    for ref in (np.exp(x), torch.exp(xt).cpu().numpy()):
        ulp = np.abs(y - ref) / np.spacing(ref)
        assert np.max(ulp) <= 2.0, (np.max(ulp), x[np.argmax(ulp)])
    assert y[2] == 1.0 and y[3] == 1.0 and y[5] == 0.5


def test_emulated_predict(cuda, oracle, cm_features):
    rng = np.random.default_rng(4)
    Xtr, Xte = cm_features[:900], cm_features[900:]
    alpha = rng.normal(size=900)
    Ks = oracle.gaussian_kernel(Xtr, Xte, 1000.0)
    expect = Ks.T @ alpha
    args = (torch.from_numpy(Xtr).to(cuda), torch.from_numpy(Xte).to(cuda), 1000.0,
            torch.from_numpy(alpha).to(cuda))
    y = core.predict("gaussian", *args, emulated=True).cpu().numpy()
    scale = np.abs(Ks.T) @ np.abs(alpha)
    assert np.max(np.abs(y - expect) / scale) <= 1e-12
    assert np.array_equal(y, core.predict("gaussian", *args, emulated=True).cpu().numpy())


@pytest.mark.parametrize("sigma", [100.0, 1000.0, 10 ** 4.2])
def test_fixed_point_laplacian(cuda, oracle, cm_features, sigma):
    # exact integer L1 sums: within 1e-12 of the oracle, exactly symmetric
    X = cm_features
    A, B = X[:700], X[700:]
    At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    K = core.kernel_matrix("laplacian", At, Bt, sigma, emulated=True).cpu().numpy()
    assert relerr(K, oracle.laplacian_kernel(A, B, sigma)) <= RTOL
    Ks = core.kernel_matrix("laplacian", At, At, sigma, symmetric=True, emulated=True).cpu().numpy()
    assert np.array_equal(Ks, Ks.T)
    assert relerr(Ks, oracle.laplacian_kernel(A, A, sigma)) <= RTOL


def test_fixed_point_laplacian_reference_test_and_fallback(cuda, oracle):
    # tests/test_kernels.py:34-63 (sigma = 100, fixed point) and sigma = 1, where the
    # fixed-point bound d * 2^-F / sigma is not met and the FP64 kernel runs
    g = load_golden("kernels_seed666.npz")
    X, Xs = g["X"], g["Xs"]
    for s in (float(g["sigma"]), 1.0):
        K = core.kernel_matrix("laplacian", torch.from_numpy(X).to(cuda),
                               torch.from_numpy(Xs).to(cuda), s, emulated=True).cpu().numpy()
        assert relerr(K, oracle.laplacian_kernel(X, Xs, s)) <= RTOL
        if s == float(g["sigma"]):
            assert np.allclose(K, g["laplacian"])


def test_more_kernels_reference_tests(cuda, oracle):
    # tests/test_kernels.py:93-214 through the drop-in API: the reference test's own
    # expectations (allclose) and the oracle (1e-12), plus the symmetric K(X, X)
    g = load_golden("kernels_more_seed666.npz")
    inp = more_kernel_inputs()
    s = float(g["sigma"])
    X, Xs = inp["linear"]
    K = linear_kernel(X, Xs)
    assert K.flags.f_contiguous and K.shape == (25, 20)
    assert np.allclose(K, g["linear"]) and relerr(K, oracle.linear_kernel(X, Xs)) <= RTOL
    Ks = linear_kernel(X, X)
    assert np.array_equal(Ks, Ks.T) and relerr(Ks, oracle.linear_kernel(X, X)) <= RTOL
    for metric in ("l1", "l2"):
        for order in (0, 1, 2):
            key = "matern_%s_%d" % (metric, order)
            X, Xs = inp[key]
            K = matern_kernel(X, Xs, s, order=order, metric=metric)
            assert K.flags.f_contiguous and np.allclose(K, g[key])
            assert relerr(K, g[key]) <= RTOL
            Ks = matern_kernel(X, X, s, order=order, metric=metric)
            assert np.array_equal(Ks, Ks.T)
    for ng in (0, 1, 2):
        X, Xs = inp["sargan_%d" % ng]
        gam = inp["sargan_%d_gammas" % ng]
        K = sargan_kernel(X, Xs, s, gam)
        assert np.allclose(K, g["sargan_%d" % ng])
        assert relerr(K, oracle.sargan_kernel(X, Xs, s, gam)) <= RTOL
        Ks = sargan_kernel(X, X, s, gam)
        assert np.array_equal(Ks, Ks.T)


@pytest.mark.parametrize("na,nb", [(1, 1), (63, 65), (130, 77)])
def test_more_kernels_cm_features(cuda, oracle, cm_features, na, nb):
    # odd shapes on CM features (sigma 1000), C-order inputs through core, and the
    # symmetric one-triangle path against the oracle
    A, B = cm_features[:na], cm_features[200:200 + nb]
    At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    gam = np.array([0.7, 0.2, 0.05])
    cases = [("linear", {}, lambda a, b: oracle.linear_kernel(a, b)),
             ("sargan", {"gammas": gam}, lambda a, b: oracle.sargan_kernel(a, b, 1000.0, gam))]
    for order in (0, 1, 2):
        cases.append(("matern_l2", {"order": order},
                      lambda a, b, o=order: oracle.matern_kernel_l2(a, b, 1000.0, o)))
    for kind, kw, ofn in cases:
        K = core.kernel_matrix(kind, At, Bt, 1000.0, **kw).cpu().numpy()
        assert relerr(K, ofn(A, B)) <= RTOL, kind
        Ks = core.kernel_matrix(kind, At, At, 1000.0, symmetric=True, **kw).cpu().numpy()
        Ko = ofn(A, A)
        assert np.array_equal(Ks, Ks.T), kind
        assert relerr(Ks, Ko) <= RTOL, kind


def test_more_kernels_arguments(cuda, cm_features):
    # the C-ABI rejects a Matern order outside 0..2 and a missing gamma array; the
    # drop-in maps orders beyond 2 to the Fortran's third branch, and no gammas to
    # the Laplacian kernel, like the reference wrapper
    A = cm_features[:20]
    At = torch.from_numpy(A).to(cuda)
    K = torch.empty((20, 20), dtype=torch.float64, device=cuda)
    lib = _lib.load()
    st = lib.qmlg_matern_kernel_l2(At.data_ptr(), 276, 20, At.data_ptr(), 276, 20, 276, 1000.0, 3,
                                   K.data_ptr(), 20, 0, 0.0, None)
    assert st == _lib.QMLG_E_ARG
    st = lib.qmlg_sargan_kernel(At.data_ptr(), 276, 20, At.data_ptr(), 276, 20, 276, 1000.0, None,
                                2, K.data_ptr(), 20, 0, 0.0, None)
    assert st == _lib.QMLG_E_ARG
    assert np.array_equal(matern_kernel(A, A[:7], 1000.0, order=3, metric="l2"),
                          matern_kernel(A, A[:7], 1000.0, order=2, metric="l2"))
    assert np.array_equal(sargan_kernel(A, A[:7], 1000.0, []), laplacian_kernel(A, A[:7], 1000.0))
    with pytest.raises(SystemExit):
        matern_kernel(A, A, 1000.0, order=3, metric="l1")
    with pytest.raises(SystemExit):
        matern_kernel(A, A, 1000.0, metric="l3")


@pytest.mark.parametrize("persistent", [1, 0])
def test_emulated_tiles_across_bands(cuda, oracle, persistent):
    # The tensor-core kernels visit their tiles in bands of 1024 i-rows.  Sizes
    # spanning several bands, with a persistent grid and with one CTA per tile:
    # entries, predictions and the trailing update against the oracle and FP64, and
    # bit-identical between the two launch shapes.
    b = generate_molecules(3700, seed=21)
    X = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    A, B = X[:2600], X[2600:]
    At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    rng = np.random.default_rng(12)
    alpha = rng.normal(size=2600)
    P = rng.normal(size=(2100, 512)) * np.exp(rng.normal(size=(2100, 1)))
    C = rng.normal(size=(2100, 2100))
    lib = core.lib()
    outs = {}
    try:
        for mode in (1, persistent):
            lib.qmlg_set_thread_persistent(mode)
            K = core.kernel_matrix("gaussian", At, Bt, 400.0, emulated=True).cpu().numpy()
            Ks = core.kernel_matrix("gaussian", At, At, 400.0, symmetric=True,
                                    emulated=True).cpu().numpy()
            y = core.predict("gaussian", At, Bt, 400.0, torch.from_numpy(alpha).to(cuda),
                             emulated=True).cpu().numpy()
            Ct = torch.from_numpy(C.copy()).to(cuda)
            core.syrk_emulated(Ct, torch.from_numpy(P).to(cuda))
            outs[mode] = (K, Ks, y, Ct.cpu().numpy())
    finally:
        lib.qmlg_set_thread_persistent(1)
    K, Ks, y, Cout = outs[persistent]
    Ko = oracle.gaussian_kernel(A, B, 400.0)
    assert relerr(K, Ko) <= RTOL
    assert np.array_equal(Ks, Ks.T)
    assert relerr(Ks, oracle.gaussian_kernel(A, A, 400.0)) <= RTOL
    assert np.max(np.abs(y - Ko.T @ alpha) / (np.abs(Ko.T) @ np.abs(alpha))) <= 1e-12
    tri = np.tril_indices(2100)
    ref = C - P @ P.T
    scale = np.abs(P) @ np.abs(P).T + np.abs(C)
    assert np.max(np.abs(Cout[tri] - ref[tri]) / scale[tri]) < 1e-14
    assert np.array_equal(np.triu(Cout, 1), np.triu(C, 1))
    for u, v in zip(outs[1], outs[persistent]):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("sigma", [10.0, 1000.0])
def test_laplacian_async_entries_match_synchronous(cuda, cm_features, sigma):
    # The capture-safe fixed-point entries decide the grid on the device: K and the
    # predictions equal the synchronous entries' bit for bit.  At sigma = 10 the
    # fixed-point bound d 2^-F / sigma <= 0.5e-12 fails for CM features, so the FP64
    # kernel launched beside the fixed-point one writes the result and 8 is flagged.
    X = cm_features
    At = torch.from_numpy(X[:700]).to(cuda)
    Bt = torch.from_numpy(X[700:]).to(cuda)
    lib = core.lib()
    stream = torch.cuda.current_stream().cuda_stream
    want_flag = 8 if sigma == 10.0 else 0
    for sym in (False, True):
        B = At if sym else Bt
        nb = B.shape[0]
        flags = _lib.QMLG_KERNEL_SYMMETRIC if sym else 0
        ref = core.kernel_matrix("laplacian", At, B, sigma, symmetric=sym, emulated=True)
        buf = torch.full((nb, 700), float("nan"), dtype=torch.float64, device=cuda)
        flag = torch.zeros(1, dtype=torch.int32, device=cuda)
        ws_bytes = lib.qmlg_laplacian_kernel_fixed_workspace_size(700, nb, 276, flags)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
        st = lib.qmlg_laplacian_kernel_fixed_async(At.data_ptr(), 276, 700, B.data_ptr(), 276, nb,
                                                   276, sigma, buf.data_ptr(), 700, flags, 0.0,
                                                   flag.data_ptr(), ws.data_ptr(), ws_bytes, stream)
        assert st == 0
        torch.cuda.synchronize()
        assert torch.equal(buf.T, ref)
        assert int(flag.item()) == want_flag
    alpha = torch.from_numpy(np.random.default_rng(2).normal(size=700)).to(cuda)
    yref = core.predict("laplacian", At, Bt, sigma, alpha, emulated=True)
    flag = torch.zeros(1, dtype=torch.int32, device=cuda)
    y = core.predict_laplacian_async(At, Bt, sigma, alpha, flag)
    torch.cuda.synchronize()
    assert torch.equal(y, yref)
    assert int(flag.item()) == want_flag


def linear_emulated_tolerance(A, B):
    # the documented bound, |K - A B^T| <= 2^(eA + eB - 56) kp 9/4 with 2^eA > max|a_j|
    # and 2^eB > max|b_i| of the two rows, plus the oracle's own FP64 rounding
    kp = -(-A.shape[1] // 64) * 64
    ea = np.frexp(np.max(np.abs(A), axis=1))[1]
    eb = np.frexp(np.max(np.abs(B), axis=1))[1]
    bound = np.ldexp(1.0, ea[:, None] + eb[None, :] - 56) * kp * 9 / 4
    return bound + A.shape[1] * 2.0 ** -53 * (np.abs(A) @ np.abs(B).T)


@pytest.mark.parametrize("na,nb", [(1, 1), (63, 65), (130, 77), (300, 173)])
def test_linear_kernel_emulated(cuda, oracle, cm_features, na, nb):
    # the tensor-core linear kernel against the oracle, entry by entry within its
    # bound, on CM features and on rows whose scales span twelve decades
    rng = np.random.default_rng(na * 1000 + nb)
    scaled = rng.standard_normal((na + nb, 45)) * 10.0 ** rng.uniform(-6, 6, (na + nb, 1))
    for A, B in ((cm_features[:na], cm_features[300:300 + nb]), (scaled[:na], scaled[na:])):
        At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
        K = core.kernel_matrix("linear", At, Bt, 1.0, emulated=True).cpu().numpy()
        Ko = oracle.linear_kernel(A, B)
        assert np.all(np.abs(K - Ko) <= linear_emulated_tolerance(A, B))
        Ks = core.kernel_matrix("linear", At, At, 1.0, symmetric=True, diag_shift=0.5,
                                emulated=True).cpu().numpy()
        Kso = oracle.linear_kernel(A, A) + 0.5 * np.eye(na)
        assert np.array_equal(Ks, Ks.T)
        assert np.all(np.abs(Ks - Kso) <= linear_emulated_tolerance(A, A) + 2.0 ** -53)
    # CM features: within 1e-12 of the largest entry
    A, B = cm_features[:na], cm_features[300:300 + nb]
    K = core.kernel_matrix("linear", torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda),
                           1.0, emulated=True).cpu().numpy()
    Ko = oracle.linear_kernel(A, B)
    assert np.max(np.abs(K - Ko)) <= 1e-12 * np.max(np.abs(Ko))


def test_linear_kernel_emulated_non_finite_and_reference(cuda, oracle):
    # input that is not finite goes to the FP64 kernel (the same NaN/inf pattern);
    # the reference test's inputs give its expectations
    g = load_golden("kernels_more_seed666.npz")
    X, Xs = more_kernel_inputs()["linear"]
    Xt, Xst = torch.from_numpy(X).to(cuda), torch.from_numpy(Xs).to(cuda)
    K = core.kernel_matrix("linear", Xt, Xst, 1.0, emulated=True).cpu().numpy()
    assert np.allclose(K, g["linear"])
    assert np.all(np.abs(K - oracle.linear_kernel(X, Xs)) <= linear_emulated_tolerance(X, Xs))
    Xbad = X.copy()
    Xbad[3, 2] = np.inf
    Xbad[5, 0] = np.nan
    Xb = torch.from_numpy(Xbad).to(cuda)
    Ke = core.kernel_matrix("linear", Xb, Xst, 1.0, emulated=True).cpu().numpy()
    Kf = core.kernel_matrix("linear", Xb, Xst, 1.0).cpu().numpy()
    assert np.array_equal(Ke, Kf, equal_nan=True)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("na,nb", [(1, 1), (63, 65), (300, 173)])
def test_matern_kernel_emulated(cuda, oracle, cm_features, order, na, nb):
    # Matern L2 orders 1 and 2 on the tensor cores: within 1e-12 relative per entry,
    # exactly symmetric, the shifted diagonal, and rows a hair apart (d near 0)
    A, B = cm_features[:na], cm_features[300:300 + nb]
    near = A + np.random.default_rng(na).standard_normal(A.shape) * 1e-7
    At, Bt, Nt = (torch.from_numpy(x).to(cuda) for x in (A, B, near))
    for sigma in (1000.0, 250.0):
        K = core.kernel_matrix("matern_l2", At, Bt, sigma, order=order, emulated=True)
        assert relerr(K.cpu().numpy(), oracle.matern_kernel_l2(A, B, sigma, order)) <= RTOL
        Kn = core.kernel_matrix("matern_l2", At, Nt, sigma, order=order, emulated=True)
        assert relerr(Kn.cpu().numpy(), oracle.matern_kernel_l2(A, near, sigma, order)) <= RTOL
        Ks = core.kernel_matrix("matern_l2", At, At, sigma, order=order, symmetric=True,
                                diag_shift=0.5, emulated=True).cpu().numpy()
        assert np.array_equal(Ks, Ks.T)
        assert relerr(Ks, oracle.matern_kernel_l2(A, A, sigma, order) + 0.5 * np.eye(na)) <= RTOL


def test_matern_kernel_emulated_falls_back(cuda, cm_features):
    # order 0, a sigma too small for the digit bound, and non-finite input take the
    # FP64 kernel: the same bits as emulated=False
    A = cm_features[:70].copy()
    At = torch.from_numpy(A).to(cuda)
    bad = A.copy()
    bad[4, 7] = np.nan
    Bt = torch.from_numpy(bad).to(cuda)
    for X, Y, sigma, order in ((At, At, 1000.0, 0), (At, At, 1.0, 2), (At, Bt, 1000.0, 1)):
        Ke = core.kernel_matrix("matern_l2", X, Y, sigma, order=order, emulated=True)
        Kf = core.kernel_matrix("matern_l2", X, Y, sigma, order=order)
        assert np.array_equal(Ke.cpu().numpy(), Kf.cpu().numpy(), equal_nan=True)


@pytest.mark.parametrize("na,nb", [(1, 1), (63, 65), (300, 173)])
def test_sargan_kernel_fixed(cuda, oracle, cm_features, na, nb):
    # the Sargan kernel from exact fixed-point L1 sums: within 1e-12 relative per entry
    # for gammas >= 0, exactly symmetric with a shifted diagonal
    A, B = cm_features[:na], cm_features[300:300 + nb]
    At, Bt = torch.from_numpy(A).to(cuda), torch.from_numpy(B).to(cuda)
    for gam in ([], [0.7], [0.7, 0.2, 0.05]):
        for sigma in (1000.0, 500.0):
            K = core.kernel_matrix("sargan", At, Bt, sigma, gammas=gam, emulated=True)
            assert relerr(K.cpu().numpy(), oracle.sargan_kernel(A, B, sigma, gam)) <= RTOL
            Ks = core.kernel_matrix("sargan", At, At, sigma, gammas=gam, symmetric=True,
                                    diag_shift=0.5, emulated=True).cpu().numpy()
            assert np.array_equal(Ks, Ks.T)
            Ko = oracle.sargan_kernel(A, A, sigma, gam) + 0.5 * np.eye(na)
            assert relerr(Ks, Ko) <= RTOL


def test_sargan_kernel_fixed_falls_back(cuda, cm_features):
    # a negative gamma, a sigma too small for the grid's bound and NaN input take the
    # FP64 kernel: the same bits as emulated=False
    A = cm_features[:70].copy()
    At = torch.from_numpy(A).to(cuda)
    bad = A.copy()
    bad[4, 7] = np.nan
    Bt = torch.from_numpy(bad).to(cuda)
    for Y, sigma, gam in ((At, 1000.0, [0.7, -0.2]), (At, 1e-3, [0.5]), (Bt, 1000.0, [0.5])):
        Ke = core.kernel_matrix("sargan", At, Y, sigma, gammas=gam, emulated=True).cpu().numpy()
        Kf = core.kernel_matrix("sargan", At, Y, sigma, gammas=gam).cpu().numpy()
        assert np.array_equal(Ke, Kf, equal_nan=True)
    # a NaN in B alone reaches the fixed-point Laplacian's FP64 fallback too
    Ke = core.kernel_matrix("laplacian", At, Bt, 1000.0, emulated=True).cpu().numpy()
    Kf = core.kernel_matrix("laplacian", At, Bt, 1000.0).cpu().numpy()
    assert np.array_equal(Ke, Kf, equal_nan=True)


def test_laplacian_fixed_predict_nan_falls_back(cuda, cm_features):
    # a NaN in the test rows alone takes the fused FP64 prediction: the same bits
    Xtr = torch.from_numpy(cm_features[:200].copy()).to(cuda)
    bad = cm_features[200:260].copy()
    bad[3, 11] = np.nan
    Xte = torch.from_numpy(bad).to(cuda)
    alpha = torch.linspace(-1.0, 1.0, 200, dtype=torch.float64, device=cuda)
    ye = core.predict("laplacian", Xtr, Xte, 1000.0, alpha, emulated=True).cpu().numpy()
    yf = core.predict("laplacian", Xtr, Xte, 1000.0, alpha).cpu().numpy()
    assert np.isnan(ye[3]) and np.array_equal(ye, yf, equal_nan=True)
