"""The C-ABI library builds, loads and exports every symbol include/qmlg.h declares
(no GPU needed: nothing is called but the version string)."""
import os
import re

from conftest import ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "qmlg.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qmlg_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for name in ("qmlg_coulomb_matrix", "qmlg_gaussian_kernel", "qmlg_laplacian_kernel",
                 "qmlg_solve", "qmlg_cholesky", "qmlg_predict_fused"):
        assert name in syms


def test_library_exports_every_declared_symbol():
    from qml_gb300 import _lib
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name
    assert b"sm_103a" in lib.qmlg_version()


def test_no_cpu_fallback():
    # without a GPU the product path refuses to run instead of computing on the host
    import numpy as np
    import pytest
    import torch

    from qml_gb300 import core
    from qml_gb300.kernels import gaussian_kernel
    from qml_gb300.math import cho_solve

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X = torch.rand(10, 276, dtype=torch.float64)
    with pytest.raises(TypeError):
        core.kernel_matrix("gaussian", X, X, 1000.0)
    with pytest.raises(RuntimeError):
        gaussian_kernel(np.random.rand(5, 276), np.random.rand(4, 276), 100.0)
    A = np.eye(4) * 2.0
    with pytest.raises(RuntimeError):
        cho_solve(A, np.ones(4))
