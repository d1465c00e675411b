"""End-to-end KRR on the GPU (molecules -> CM -> K -> solve -> predict) against the
oracle pipeline on the same synthetic molecules."""
import numpy as np
import pytest
import torch

from qml_gb300 import core
from qml_gb300.krr import KRR, molecules_to_device
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel,sigma,lam", [("gaussian", 1000.0, 1e-8), ("laplacian", 10 ** 4.2, 1e-10)])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_krr_pipeline(cuda, oracle, kernel, sigma, lam, precision):
    b = generate_molecules(2000, seed=17)
    ntr = 1000
    z, r, off = molecules_to_device(b)
    X = core.coulomb_matrix_batch(z, r, off, 23)
    y = torch.from_numpy(b.labels).to(cuda)
    model = KRR(kernel=kernel, sigma=sigma, lam=lam, precision=precision).fit(X[:ntr], y[:ntr])
    yhat = model.predict(X[ntr:]).cpu().numpy()

    Xo = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    assert np.array_equal(X.cpu().numpy(), Xo)
    kfn = oracle.gaussian_kernel if kernel == "gaussian" else oracle.laplacian_kernel
    K = np.ascontiguousarray(kfn(Xo[:ntr], Xo[:ntr], sigma))
    alpha = oracle.refined_solve(K, b.labels[:ntr], lam)
    Ks = kfn(Xo[:ntr], Xo[ntr:], sigma)
    yo = Ks.T @ alpha
    # alpha itself is compared in test_gpu_solve on identical K; here the kernels may
    # differ in the last bits, which cond(K + lambda I) amplifies, so compare the
    # predictions (well conditioned) and the test error
    assert np.max(np.abs(yhat - yo)) < 1e-6 * np.max(np.abs(yo)) + 1e-6
    mae_gpu = np.mean(np.abs(yhat - b.labels[ntr:]))
    mae_ref = np.mean(np.abs(yo - b.labels[ntr:]))
    assert abs(mae_gpu - mae_ref) < 1e-6 * mae_ref
    assert model.report["status"] == 0
