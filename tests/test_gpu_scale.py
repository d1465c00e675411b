"""Parity at the benchmark sizes, against the oracle.

* 20000 training x 5000 test molecules (the "kernel and solve at scale" size):
  every Coulomb matrix bit for bit; every entry of the tensor-core Gaussian K and of
  the fixed-point Laplacian K within 1e-12 of the oracle's FP64 kernels; the mixed
  alpha within 1e-8 of the oracle's refined solve of the same FP64 K for
  lambda in {1e-4, 1e-6, 1e-8}, and the FP64 path's refined alpha within 1e-12; the
  predictions within 1e-12 of sum_j |k_ij alpha_j| when alpha is shared, and the
  test MAE of the whole GPU pipeline beside the oracle pipeline's.
* Batched fits of 500..8000 molecules recorded into one CUDA graph, all three
  lambdas: alpha within 1e-8 of the refined oracle on each fit's own K.
* A resident 50000-molecule serving model: queries alone and in the mix agree bit
  for bit and match the oracle's prediction with the same alpha.
* 60000 training molecules (a 28.8 GB K), Gaussian and Laplacian: sampled rows of K
  against the oracle, and the backward error of alpha on sampled rows, with the
  residual summed in double-double by the oracle from the GPU's own K.

The oracle's K and refined solves at these sizes take tens of seconds on the host
cores; each fixture computes them once per module.
"""
import numpy as np
import pytest
import torch

from qml_gb300 import core
from qml_gb300.krr import KRR, molecules_to_device
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu

NTR, NTE, SIGMA = 20000, 5000, 1000.0


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def at_scale(oracle, cuda):
    b = generate_molecules(NTR + NTE, seed=2024)
    Xo = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    z, r, off = molecules_to_device(b)
    X = core.coulomb_matrix_batch(z, r, off, 23)
    Kg = np.ascontiguousarray(oracle.gaussian_kernel(Xo[:NTR], Xo[:NTR], SIGMA))
    return {"batch": b, "Xo": Xo, "X": X, "Kg": Kg, "refined": {}}


def refined(oracle, at_scale, lam):
    cache = at_scale["refined"]
    if lam not in cache:
        cache[lam] = oracle.refined_solve(at_scale["Kg"], at_scale["batch"].labels[:NTR], lam)
    return cache[lam]


def test_cm_25000_bit_exact(at_scale):
    assert np.array_equal(at_scale["X"].cpu().numpy(), at_scale["Xo"])


def test_tensor_core_gaussian_K_20000(at_scale):
    X = at_scale["X"]
    K = core.kernel_matrix("gaussian", X[:NTR], X[:NTR], SIGMA, symmetric=True,
                           emulated=True).cpu().numpy()
    Ko = at_scale["Kg"]  # row-major copy of the (symmetric) Fortran-ordered oracle K
    assert np.max(np.abs(K - Ko) / Ko) <= 1e-12
    assert np.array_equal(K, K.T)


def test_fixed_point_laplacian_K_20000(at_scale, oracle):
    X, Xo = at_scale["X"], at_scale["Xo"]
    K = core.kernel_matrix("laplacian", X[:NTR], X[:NTR], SIGMA, symmetric=True,
                           emulated=True).cpu().numpy()
    Ko = oracle.laplacian_kernel(Xo[:NTR], Xo[:NTR], SIGMA)
    assert np.max(np.abs(K - Ko) / Ko) <= 1e-12
    assert np.array_equal(K, K.T)


@pytest.mark.parametrize("lam", [1e-4, 1e-6, 1e-8])
def test_mixed_alpha_20000_vs_refined_oracle(at_scale, oracle, cuda, lam):
    xr = refined(oracle, at_scale, lam)
    y = at_scale["batch"].labels[:NTR]
    x, rep = core.solve(torch.from_numpy(at_scale["Kg"]).to(cuda), torch.from_numpy(y).to(cuda),
                        lam, precision="mixed")
    assert rep["status"] == 0 and rep["fell_back"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-8, rep


def test_fp64_alpha_20000_vs_refined_oracle(at_scale, oracle, cuda):
    lam = 1e-8
    xr = refined(oracle, at_scale, lam)
    y = at_scale["batch"].labels[:NTR]
    x, rep = core.solve(torch.from_numpy(at_scale["Kg"]).to(cuda), torch.from_numpy(y).to(cuda),
                        lam, precision="fp64")
    assert rep["status"] == 0, rep
    assert rel(x.cpu().numpy(), xr) <= 1e-12, rep


def test_predictions_and_pipeline_20000(at_scale, oracle, cuda):
    lam = 1e-8
    b, Xo, X = at_scale["batch"], at_scale["Xo"], at_scale["X"]
    y = torch.from_numpy(b.labels).to(cuda)
    # the whole GPU pipeline: tensor-core K, mixed solve, tensor-core prediction
    model = KRR(sigma=SIGMA, lam=lam, precision="mixed").fit(X[:NTR], y[:NTR])
    yhat = model.predict(X[NTR:]).cpu().numpy()
    alpha = model.alpha.cpu().numpy()
    # with alpha shared, the prediction is within 1e-12 of sum_j |k_ij alpha_j|
    Ks = oracle.gaussian_kernel(Xo[:NTR], Xo[NTR:], SIGMA)
    expect = Ks.T @ alpha
    scale = np.abs(Ks.T) @ np.abs(alpha)
    assert np.max(np.abs(yhat - expect) / scale) <= 1e-12
    # the oracle pipeline (oracle K, refined solve, oracle Ks): the two pipelines'
    # kernels differ in the last bits, which cond(K + lambda I) ~ 1e12 amplifies in
    # alpha, not in the predictions' quality
    yo = Ks.T @ refined(oracle, at_scale, lam)
    mae_gpu = float(np.mean(np.abs(yhat - b.labels[NTR:])))
    mae_ref = float(np.mean(np.abs(yo - b.labels[NTR:])))
    diff = float(np.max(np.abs(yhat - yo)))
    print("20000 x 5000 Gaussian, lambda 1e-8: MAE GPU %.9f, oracle %.9f, max |dy| %.3e"
          % (mae_gpu, mae_ref, diff))
    assert abs(mae_gpu - mae_ref) <= 1e-6 * mae_ref, (mae_gpu, mae_ref, diff)


def test_laplacian_prediction_20000(at_scale, oracle, cuda):
    Xo, X = at_scale["Xo"], at_scale["X"]
    rng = np.random.default_rng(3)
    alpha = rng.normal(size=NTR) * np.exp(rng.normal(size=NTR) * 3)
    a = torch.from_numpy(alpha).to(cuda)
    yhat = core.predict("laplacian", X[:NTR], X[NTR:], SIGMA, a, emulated=True).cpu().numpy()
    Ks = oracle.laplacian_kernel(Xo[:NTR], Xo[NTR:], SIGMA)
    scale = np.abs(Ks.T) @ np.abs(alpha)
    assert np.max(np.abs(yhat - Ks.T @ alpha) / scale) <= 1e-12


# ------------------------------------------------- batched fits up to 8000 --

def test_batched_fits_up_to_8000(oracle, cuda):
    from qml_gb300.batch import BatchedKRR, Problem
    pool = generate_molecules(9000, seed=405)
    Xo = oracle.cm_sorted_batch(pool.charges, pool.coordinates, pool.offsets, 23)
    X = torch.from_numpy(Xo).to(cuda)
    y = torch.from_numpy(pool.labels).to(cuda)
    spec = [(8000, 1000.0, 1e-8), (5000, 250.0, 1e-6), (3000, 2000.0, 1e-4),
            (6500, 500.0, 1e-8), (1200, 1000.0, 1e-6), (500, 2000.0, 1e-8)]
    probs, starts = [], []
    for k, (n, s, lam) in enumerate(spec):
        st = (k * 331) % (9000 - n + 1)
        starts.append(st)
        probs.append(Problem(X[st:st + n].contiguous(), y[st:st + n].contiguous(), s, lam))
    b = BatchedKRR(probs, refine_steps=3, streams=3)
    b.capture()
    b.replay()
    alphas, reps = b.results()
    for i, ((n, s, lam), st) in enumerate(zip(spec, starts)):
        assert reps[i]["info"] == 0 and reps[i]["flags"] == 0, reps[i]
        F = b.K[i].cpu().numpy()
        U = np.triu(F, 1)
        K = U + U.T + np.eye(n)  # the fit's own K (the diagonal of a Gaussian K is 1)
        Ko = oracle.gaussian_kernel(Xo[st:st + n], Xo[st:st + n], s)
        assert np.max(np.abs(K - Ko) / Ko) <= 1e-12
        ref = oracle.refined_solve(K, pool.labels[st:st + n], lam)
        assert rel(alphas[i].cpu().numpy(), ref) <= 1e-8, (n, s, lam, reps[i])


# ---------------------------------------------- 50000-molecule serving model --

def test_serving_resident_50000(oracle, cuda):
    from qml_gb300 import serving
    ntr = 50000
    train = generate_molecules(ntr, seed=2031)
    z, r, o = molecules_to_device(train)
    X = core.coulomb_matrix_batch(z, r, o, 23)
    y = torch.from_numpy(train.labels).to(cuda)
    model = KRR(sigma=1000.0, lam=1e-8, precision="mixed").fit(X, y)
    assert model.report["status"] == 0 and model.report["fell_back"] == 0, model.report
    ex = serving.GpuExecutor(n_streams=4)
    ex.add_model("main", X, model.alpha, 1000.0)
    pool = generate_molecules(8000, seed=2032)
    reqs = serving.poisson_workload(300.0, 0.6, pool, "main", fit_every=60, fit_sizes=(1000, 3000),
                                    seed=9, max_query=4096)
    done = serving.Server(ex, serving.Scheduler(budget_bytes=48 << 30, max_slots=4,
                                                model_sizes={"main": ntr})).run(reqs)
    assert len(done) == len(reqs) and all(r.error is None for r in done)
    preds = [r for r in done if r.kind == "predict"]
    assert len(preds) > 20
    Xo = oracle.cm_sorted_batch(train.charges, train.coordinates, train.offsets, 23)
    alpha = model.alpha.cpu().numpy()
    for req in preds[:6]:
        alone = serving.Request(-1, "predict", "main", req.charges, req.coordinates, req.offsets, 0.0)
        ev, finish = ex.launch_predict([alone])
        ev.synchronize()
        finish()
        assert np.array_equal(alone.result, req.result)
        Xq = oracle.cm_sorted_batch(req.charges, req.coordinates, req.offsets, 23)
        Ks = oracle.gaussian_kernel(Xo, Xq, 1000.0)
        scale = np.abs(Ks.T) @ np.abs(alpha)
        assert np.max(np.abs(req.result - Ks.T @ alpha) / scale) <= 1e-12


# ------------------------------------------------------- 60000 training rows --

@pytest.mark.parametrize("kind", ["gaussian", "laplacian"])
def test_60000_sampled_rows_and_backward_error(oracle, cuda, kind):
    ntr, lam = 60000, 1e-8
    b = generate_molecules(ntr, seed=2029)
    z, r, off = molecules_to_device(b)
    X = core.coulomb_matrix_batch(z, r, off, 23)
    y = b.labels
    K = core.kernel_matrix(kind, X, X, SIGMA, symmetric=True, emulated=True)
    rows = np.sort(np.random.default_rng(11).choice(ntr, size=48, replace=False))
    ri = torch.from_numpy(rows).to(cuda)
    Krows = K[ri].cpu().numpy()  # (48, ntr), before the factorisation
    Xo = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    kfn = oracle.gaussian_kernel if kind == "gaussian" else oracle.laplacian_kernel
    Ko = kfn(Xo[rows], Xo, SIGMA)  # (48, ntr) Fortran order
    assert np.max(np.abs(Krows - Ko) / Ko) <= 1e-12
    x, rep = core.solve(K, torch.from_numpy(y).to(cuda), lam, precision="mixed")
    assert rep["status"] == 0 and rep["fell_back"] == 0, rep
    # K is the column-major matrix the solve factorised in its upper triangle, so
    # row i keeps its K values left of the diagonal
    for k, i in enumerate(rows[-4:]):
        i = int(i)
        assert np.array_equal(K[i, :i].cpu().numpy(), Krows[len(rows) - 4 + k, :i])
    xs = x.cpu().numpy()
    # the residual of the sampled rows, summed in double-double by the oracle from the
    # GPU's own K: alpha solves a system within FP64 rounding of (K + lambda I)
    r_rows = oracle.rows_residual_dd(Krows, xs, y[rows]) - lam * xs[rows]
    scale = np.abs(Krows) @ np.abs(xs) + lam * np.abs(xs[rows]) + np.abs(y[rows])
    berr = float(np.max(np.abs(r_rows) / scale))
    print("60000 %s, lambda 1e-8: sampled-row backward error %.3e, refinement steps %d"
          % (kind, berr, rep["outer_iterations"]))
    assert berr <= 1e-15, berr
