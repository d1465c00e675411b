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


def test_xyz_ingestion_and_model_file(cuda, oracle, tmp_path):
    # XYZ files -> one ragged batch on the device -> Coulomb matrices (bit-exact vs
    # the oracle); a fitted model saved and loaded predicts bit for bit the same
    from test_io import write_fixture_xyz
    from qml_gb300.io import xyz_to_device
    from qml_gb300.krr import KRR
    paths, z, r, off = write_fixture_xyz(tmp_path)
    zt, rt, ot = xyz_to_device(paths)
    X = core.coulomb_matrix_batch(zt, rt, ot, 17).cpu().numpy()
    Xo = oracle.cm_sorted_batch(z, r, off, 17)
    assert np.array_equal(X, Xo)
    b = generate_molecules(600, seed=5)
    zb, rb, ob = molecules_to_device(b)
    Xb = core.coulomb_matrix_batch(zb, rb, ob, 23)
    y = torch.from_numpy(b.labels).to(cuda)
    m = KRR(sigma=1000.0, lam=1e-8).fit(Xb[:500], y[:500])
    path = str(tmp_path / "krr.npz")
    m.save(path)
    m2 = KRR.load(path)
    assert torch.equal(m2.predict(Xb[500:]), m.predict(Xb[500:]))
