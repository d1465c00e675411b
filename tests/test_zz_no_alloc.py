"""qmlg_predict_fused_noalloc: the prediction entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (for example a serving process
whose memory manager owns every device allocation after start-up).  Its scratch is a
fixed array inside the library, so this test calls it through the C ABI and checks
it against qmlg_predict_fused, which takes a caller workspace, on two calls in a row
(the second call reuses the array the first one left behind).  The file is named to
be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from qml_gb300 import _lib
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the same bound the fused-prediction tests use


def _call_both(lib, kind, Xtr, Xte, sigma, alpha, stream):
    ntr, d = Xtr.shape
    nte = Xte.shape[0]
    y_ws = torch.empty(nte, dtype=torch.float64, device=Xtr.device)
    y_na = torch.full((nte,), float("nan"), dtype=torch.float64, device=Xtr.device)
    ws_bytes = lib.qmlg_predict_workspace_size(ntr, nte)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=Xtr.device)
    st = lib.qmlg_predict_fused(kind, Xtr.data_ptr(), d, ntr, Xte.data_ptr(), d, nte, d, sigma,
                                alpha.data_ptr(), y_ws.data_ptr(), ws.data_ptr(), ws_bytes, stream)
    assert st == 0
    st = lib.qmlg_predict_fused_noalloc(kind, Xtr.data_ptr(), d, ntr, Xte.data_ptr(), d, nte, d,
                                        sigma, alpha.data_ptr(), y_na.data_ptr(), stream)
    assert st == 0
    torch.cuda.synchronize()
    return y_ws.cpu().numpy(), y_na.cpu().numpy()


@pytest.mark.parametrize("kind", [_lib.QMLG_KIND_GAUSSIAN, _lib.QMLG_KIND_LAPLACIAN])
def test_noalloc_matches_workspace_version_twice(kind):
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    lib = _lib.load()
    from oracle import oracle
    b = generate_molecules(1300, seed=77)
    X = oracle.cm_sorted_batch(b.charges, b.coordinates, b.offsets, 23)
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(8)
    shapes = [(1000, 300), (700, 41)]  # second call: different sizes over the same array
    for ntr, nte in shapes:
        Xtr = torch.from_numpy(X[:ntr].copy()).to(dev)
        Xte = torch.from_numpy(X[1300 - nte:].copy()).to(dev)
        alpha = torch.from_numpy(rng.normal(size=ntr)).to(dev)
        y_ws, y_na = _call_both(lib, kind, Xtr, Xte, 1000.0, alpha, stream)
        scale = np.max(np.abs(y_ws)) + 1e-300
        assert np.all(np.isfinite(y_na))
        assert np.max(np.abs(y_na - y_ws)) <= TOL * scale


@pytest.mark.parametrize("ntr,nte", [(64 * 4097, 1025),  # 4097 * 1025 partial sums > 4194304
                                      (1, 4194305)])      # one test molecule past the limit
def test_noalloc_rejects_oversized_problem(ntr, nte):
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    lib = _lib.load()
    dev = torch.device("cuda")
    d = 1
    Xtr = torch.zeros((ntr, d), dtype=torch.float64, device=dev)
    Xte = torch.zeros((nte, d), dtype=torch.float64, device=dev)
    alpha = torch.zeros(ntr, dtype=torch.float64, device=dev)
    y = torch.zeros(nte, dtype=torch.float64, device=dev)
    st = lib.qmlg_predict_fused_noalloc(_lib.QMLG_KIND_GAUSSIAN, Xtr.data_ptr(), d, ntr,
                                        Xte.data_ptr(), d, nte, d, 1.0, alpha.data_ptr(),
                                        y.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == _lib.QMLG_E_TOO_LARGE


def test_noalloc_at_the_limit_with_65536_test_tiles():
    # one training row and 4194304 test rows: exactly the array's capacity, and
    # 65536 tiles of test rows (one more than a second grid dimension could hold)
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    lib = _lib.load()
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device=dev).manual_seed(5)
    ntr, nte, d = 1, 4194304, 2
    Xtr = torch.rand((ntr, d), dtype=torch.float64, device=dev, generator=gen)
    Xte = torch.rand((nte, d), dtype=torch.float64, device=dev, generator=gen)
    alpha = torch.full((ntr,), 0.75, dtype=torch.float64, device=dev)
    for kind in (_lib.QMLG_KIND_GAUSSIAN, _lib.QMLG_KIND_LAPLACIAN):
        y_ws, y_na = _call_both(lib, kind, Xtr, Xte, 0.5, alpha, stream)
        assert np.all(np.isfinite(y_na))
        assert np.max(np.abs(y_na - y_ws)) <= TOL * np.max(np.abs(y_ws))
        # and against the closed form of the single-row sum
        diff = (Xte - Xtr).cpu().numpy()
        ref = 0.75 * (np.exp(-0.5 / 0.25 * np.sum(diff * diff, axis=1))
                      if kind == _lib.QMLG_KIND_GAUSSIAN else np.exp(-np.sum(np.abs(diff), axis=1) / 0.5))
        assert np.max(np.abs(y_na - ref)) <= 1e-12
