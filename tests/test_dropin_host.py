"""Argument checks of the drop-in API, on the host (no GPU): the same exceptions and
messages as the reference (qml/math.py:33-164, qml/representations.py:69-230), raised
before any device work."""
import numpy as np
import pytest

from qml_gb300 import math as qm
from qml_gb300 import representations as qr


@pytest.mark.parametrize("fn", [qm.cho_invert, qm.bkf_invert])
def test_inverse_needs_a_square_matrix(fn):
    with pytest.raises(ValueError, match="expected square matrix"):
        fn(np.ones((3, 4)))


@pytest.mark.parametrize("fn", [qm.cho_solve, qm.bkf_solve])
def test_solve_shape_checks(fn):
    with pytest.raises(ValueError, match="expected square matrix"):
        fn(np.ones((3, 4)), np.ones(3))
    with pytest.raises(ValueError, match="expected matrix and vector of same stride size"):
        fn(np.eye(3), np.ones(4))


@pytest.mark.parametrize("fn", [qr.generate_coulomb_matrix, qr.generate_atomic_coulomb_matrix])
def test_unknown_sorting_exits(fn, capsys):
    with pytest.raises(SystemExit):
        fn(np.array([1, 1]), np.zeros((2, 3)), size=3, sorting="bogus")
    assert "Unknown sorting scheme requested" in capsys.readouterr().out
