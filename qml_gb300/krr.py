"""Kernel-ridge regression on the GPU: the fit + predict recipe of the reference's
tests and tutorial (tests/test_energy_krr_cmat.py:66-113, docs/source/tutorial.rst:128-166):

    X  = sorted Coulomb matrices        (qmlg_coulomb_matrix)
    K  = kernel(X, X)                     (symmetric kernel)
    alpha = solve(K + lambda I, y)        (qmlg_solve, "fp64" or "mixed")
    yhat  = kernel(Xs, X) alpha           (fused prediction, Ks never materialised)

precision "fp64" runs the plain FP64 kernels and factorisation; "mixed" forms the
Gaussian contractions and the Cholesky trailing updates as emulated-FP64 products
on the bf16 tensor cores (each kernel entry within 1e-12 of FP64) and refines
alpha on the exactly summed residual.

All tensors stay in HBM; ``KRR`` keeps the training representations and alpha
resident so that predictions reuse them.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import torch

from . import core


@dataclass
class KRR:
    kernel: str = "gaussian"
    sigma: float = 1000.0
    lam: float = 1e-8
    precision: str = "mixed"
    max_outer: int = 10
    tol: float = 1e-14
    X: Optional[torch.Tensor] = None
    alpha: Optional[torch.Tensor] = None
    report: dict = field(default_factory=dict)
    K: Optional[torch.Tensor] = None

    def fit(self, X: torch.Tensor, y: torch.Tensor, keep_kernel: bool = False) -> "KRR":
        """X (n, d) float64 CUDA, y (n,) float64 CUDA."""
        emulated = self.precision == "mixed"
        K = core.kernel_matrix(self.kernel, X, X, self.sigma, symmetric=True, emulated=emulated)
        # lambda goes to the solver (the kernel's own diagonal stays exact)
        alpha, rep = core.solve(K, y, self.lam, precision=self.precision,
                                max_outer=self.max_outer, tol=self.tol)
        self.X, self.alpha, self.report = X, alpha, rep
        self.K = K if keep_kernel else None
        return self

    def save(self, path: str) -> None:
        """Write the fitted model to one .npz file (see qml_gb300.io)."""
        from .io import save_krr
        save_krr(path, self)

    @staticmethod
    def load(path: str, device="cuda") -> "KRR":
        from .io import load_krr
        return load_krr(path, device)

    def predict(self, Xs: torch.Tensor) -> torch.Tensor:
        if self.alpha is None:
            raise RuntimeError("fit() first")
        return core.predict(self.kernel, self.X, Xs, self.sigma, self.alpha,
                            emulated=self.precision == "mixed")


def molecules_to_device(batch, device="cuda", pin=True):
    """Host MoleculeBatch -> device tensors (charges, coordinates, offsets)."""
    def t(a, dtype):
        x = torch.from_numpy(a).to(dtype)
        if pin:
            x = x.pin_memory()
        return x.to(device, non_blocking=True)
    return (t(batch.charges, torch.float64), t(batch.coordinates, torch.float64),
            t(batch.offsets, torch.int64))
