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
