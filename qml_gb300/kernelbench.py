"""Run one hot-path kernel on seeded data, for timing and profiling.

    python -m qml_gb300.kernelbench syrk  --n 8192 --k 512       # emulated trailing update
    python -m qml_gb300.kernelbench gauss --n 8192               # tensor-core Gaussian K (symmetric)
    python -m qml_gb300.kernelbench lapl  --n 8192               # fixed-point Laplacian K
    python -m qml_gb300.kernelbench predict --n 20000 --m 5000   # tensor-core fused prediction
    python -m qml_gb300.kernelbench cm    --n 25000              # sorted Coulomb matrices
    python -m qml_gb300.kernelbench factor --n 20000             # mixed Cholesky of the KRR K
    python -m qml_gb300.kernelbench solve  --n 20000             # mixed solve with refinement
    python -m qml_gb300.kernelbench krr --n 40000 --m 10000      # one mixed KRR fit + predict step
    python -m qml_gb300.kernelbench batch --m 64                 # 64 batched fits, grouped path
    python -m qml_gb300.kernelbench residual --n 20000           # exact residual y - (K + lam I) x

Each command runs the kernel `--reps` times after one warm-up call and prints the
mean time per call (CUDA events on the launching stream).  `factor` and `solve` work
on the Gaussian K (sigma, lambda = 1e-8) of seeded synthetic molecules and restore K
before every call, outside the timed region.
"""
from __future__ import annotations

import argparse
import json

import torch

from . import core
from .krr import molecules_to_device
from .synthetic import generate_molecules


def _features(n, seed):
    b = generate_molecules(n, seed=seed)
    z, r, o = molecules_to_device(b)
    return core.coulomb_matrix_batch(z, r, o, 23), (z, r, o)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("kernel", choices=["syrk", "gauss", "lapl", "predict", "cm", "factor", "solve",
                                      "krr", "batch", "residual"])
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--m", type=int, default=2048)
    p.add_argument("--k", type=int, default=512)
    p.add_argument("--sigma", type=float, default=1000.0)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--lam", type=float, default=1e-8)
    a = p.parse_args(argv)
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(7)
    if a.kernel == "syrk":
        C = torch.rand((a.n, a.n), dtype=torch.float64, device=dev, generator=g)
        P = torch.rand((a.n, a.k), dtype=torch.float64, device=dev, generator=g)
        run = lambda: core.syrk_emulated(C, P)  # noqa: E731
    elif a.kernel in ("gauss", "lapl"):
        X, _ = _features(a.n, 1)
        kind = "gaussian" if a.kernel == "gauss" else "laplacian"
        K = torch.empty((a.n, a.n), dtype=torch.float64, device=dev).T
        run = lambda: core.kernel_matrix(kind, X, X, a.sigma, symmetric=True, emulated=True,  # noqa: E731
                                         out=K)
    elif a.kernel == "predict":
        X, _ = _features(a.n + a.m, 2)
        alpha = torch.rand(a.n, dtype=torch.float64, device=dev, generator=g)
        run = lambda: core.predict("gaussian", X[:a.n], X[a.n:], a.sigma, alpha,  # noqa: E731
                                   emulated=True)
    elif a.kernel in ("factor", "solve"):
        X, _ = _features(a.n, 2024)
        K0 = torch.empty((a.n, a.n), dtype=torch.float64, device=dev).T
        core.kernel_matrix("gaussian", X, X, a.sigma, symmetric=True, emulated=True, out=K0)
        K = torch.empty_like(K0)
        y = torch.rand(a.n, dtype=torch.float64, device=dev, generator=g)
        if a.kernel == "factor":
            run = lambda: core.cholesky(K, a.lam, "mixed")  # noqa: E731
        else:
            run = lambda: core.solve(K, y, a.lam, "mixed")  # noqa: E731
        total = 0.0
        for i in range(a.reps + 1):
            K.copy_(K0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            torch.cuda.synchronize()
            if i > 0:
                total += e0.elapsed_time(e1)
        print(json.dumps({"kernel": a.kernel, "n": a.n, "ms_per_call": total / max(a.reps, 1)}))
        return
    elif a.kernel == "batch":
        # the bench's batching workload: m fits of N log-uniform in [500, 8000], sigma
        # and lambda drawn from the bench's sets, run eagerly on the grouped path
        import math

        import numpy as np

        from .batch import BatchedKRR, Problem
        rng = np.random.default_rng(2024 + 11)
        X, _ = _features(16000, 2024 + 12)
        y = torch.rand(16000, dtype=torch.float64, device=dev, generator=g)
        probs = []
        for _ in range(a.m):
            n = int(round(math.exp(rng.uniform(math.log(500), math.log(8000)))))
            s0 = int(rng.integers(0, 16000 - n + 1))
            probs.append(Problem(X[s0:s0 + n].contiguous(), y[s0:s0 + n].contiguous(),
                                 float(rng.choice([250.0, 500.0, 1000.0, 2000.0])),
                                 float(rng.choice([1e-4, 1e-6, 1e-8]))))
        b = BatchedKRR(probs, refine_steps=3, trsm_rows=64)
        run = b.run_eager
    elif a.kernel == "residual":
        # the refinement's exact residual on the Gaussian K of seeded molecules (the
        # upper triangle and the diagonal are read; x of mixed signs and magnitudes)
        X, _ = _features(a.n, 2024)
        K = torch.empty((a.n, a.n), dtype=torch.float64, device=dev).T
        core.kernel_matrix("gaussian", X, X, a.sigma, symmetric=True, emulated=True, out=K)
        diag = torch.diagonal(K).contiguous()
        x = torch.randn(a.n, dtype=torch.float64, device=dev, generator=g) * 1e6
        y = torch.rand(a.n, dtype=torch.float64, device=dev, generator=g)
        run = lambda: core.residual_dd(K, diag, a.lam, x, y)  # noqa: E731
    elif a.kernel == "krr":
        # the bench's step: CMs of n + m molecules, tensor-core K of the n training
        # ones, mixed solve, fused prediction of the m test molecules
        from .krr import KRR
        b = generate_molecules(a.n + a.m, seed=2024)
        z, r, o = molecules_to_device(b)
        y = torch.from_numpy(b.labels[:a.n]).to(dev)

        def run():
            X = core.coulomb_matrix_batch(z, r, o, 23)
            m = KRR(sigma=a.sigma, lam=a.lam, precision="mixed").fit(X[:a.n], y)
            m.predict(X[a.n:])
    else:
        _, (z, r, o) = _features(a.n, 3)
        run = lambda: core.coulomb_matrix_batch(z, r, o, 23)  # noqa: E731
    run()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"kernel": a.kernel, "n": a.n, "m": a.m, "k": a.k,
                      "ms_per_call": e0.elapsed_time(e1) / a.reps}))


if __name__ == "__main__":
    main()
