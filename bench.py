"""KRR fit+predict benchmark on one GB300 (per-rank replicas when launched with N > 1).

Workload (the mixed-precision target size): seeded synthetic molecules (QM7-like:
n_atoms ~ U{5..23}, Z in {1,6,7,8,16}), sorted Coulomb matrix size 23 (276 features,
FP64), Gaussian kernel sigma = 1000, lambda = 1e-8, 40000 training and 10000 test
molecules.  One step is one KRR fit + predict over molecules already in HBM:
    CM of 50000 molecules -> K = k(X, X) (40000^2, symmetric) -> alpha = solve(K + lambda I, y)
    -> yhat = k(Xs, X) alpha (fused, Ks not materialised)
with the solve in the mixed mode (emulated-FP64 tensor-core factor + refinement on
an exactly summed residual).  Beside it, in the same run:
  * the plain FP64 GPU path, timed --fp64-reps times (median), and the mixed alpha
    against the FP64-refined alpha on the same FP64 K;
  * 60000 train x 10000 test Gaussian and Laplacian fits (a 28.8 GB K);
  * continuous-batching serving against a resident 50000-molecule model (p50/p99);
  * 64 uneven fits recorded into one CUDA graph;
  * a bounded CPU sample of the reference's path on the host cores.

Prints ONE JSON line (rank 0); a compact "headline" object closes the line.
``--impl reference`` times the CPU path instead: the oracle's C/OpenMP restatement of
the reference's Fortran routines plus SciPy LAPACK dpotrf/dpotrs (the routines the
reference calls) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "KRR fit+predict s & p99 query latency: mixed vs FP64 on GB300 at 1e-8 rel err"
UNIT = "s"


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--ntrain", type=int, default=40000)
    p.add_argument("--ntest", type=int, default=10000)
    p.add_argument("--sigma", type=float, default=1000.0)
    p.add_argument("--lam", type=float, default=1e-8)
    p.add_argument("--kernel", default="gaussian", choices=["gaussian", "laplacian"])
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--fp64-reps", type=int, default=3,
                   help="plain FP64 GPU fit+predict repeats (0 skips the comparison)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    p.add_argument("--serve-n", type=int, default=50000, help="resident model size")
    p.add_argument("--serve-rate", type=float, default=100.0, help="query arrivals per second")
    p.add_argument("--serve-seconds", type=float, default=10.0)
    p.add_argument("--serve-fit-every", type=int, default=50, help="every k-th arrival is a fit")
    p.add_argument("--no-batching", action="store_true", help="skip the batched-fits measurement")
    p.add_argument("--batch-count", type=int, default=64)
    p.add_argument("--no-large", action="store_true",
                   help="skip the 60000 x 10000 Gaussian and Laplacian fits")
    p.add_argument("--large-train", type=int, default=60000)
    p.add_argument("--large-test", type=int, default=10000)
    p.add_argument("--no-extra", action="store_true",
                   help="skip the other kernel matrices and the atomic-CM / local-kernel / "
                        "inverse / unsorted-CM / file measurements")
    return p.parse_args(argv)


def workload_config(a):
    return {"workload": "krr-cm276-%s-fit%d-predict%d" % (a.kernel, a.ntrain, a.ntest),
            "n_train": a.ntrain, "n_test": a.ntest, "features": 276, "cm_size": 23,
            "kernel": a.kernel, "sigma": a.sigma, "lambda": a.lam, "solve": "mixed",
            "molecules": "synthetic QM7-like, seed %d" % a.seed,
            "l2": "inputs larger than L2 (K is %.1f GB)" % (8.0 * a.ntrain ** 2 / 1e9),
            "parallelism": "replicas"}


# ----------------------------------------------------------------- CPU leg --

def _kernel_fn(kind):
    from oracle import oracle
    return oracle.gaussian_kernel if kind == "gaussian" else oracle.laplacian_kernel


def cpu_cm(batch):
    from oracle import oracle
    t0 = time.perf_counter()
    X = oracle.cm_sorted_batch(batch.charges, batch.coordinates, batch.offsets, 23)
    return X, time.perf_counter() - t0


def cpu_test_side(Xtr, Xte, a, frac):
    """K_test on 1/frac of the test rows and the prediction GEMV on them, each
    scaled by frac (the rows are independent, so the work scales linearly)."""
    import numpy as np
    kfn = _kernel_fn(a.kernel)
    nte = Xte.shape[0]
    rows = max(1, nte // frac)
    t0 = time.perf_counter()
    Ks = kfn(Xtr, Xte[:rows], a.sigma)
    t_k = (time.perf_counter() - t0) * (nte / rows)
    alpha = np.random.default_rng(0).normal(size=Xtr.shape[0])
    t0 = time.perf_counter()
    _ = Ks.T @ alpha
    t_p = (time.perf_counter() - t0) * (nte / rows)
    return t_k, t_p


def cpu_baseline_sample(batch, a):
    """Bounded CPU sample (about ten seconds) of the reference's path, scaled to one
    full fit+predict: all Coulomb matrices; 1/16 of the rows of K_train and K_test
    (scaled by 16); LAPACK dpotrf + dpotrs on the leading N/2 block (scaled by 8,
    the N^3 ratio); the prediction GEMV on the sampled test rows (scaled by 16)."""
    import numpy as np
    from scipy.linalg import lapack
    kfn = _kernel_fn(a.kernel)
    ntr, nte = a.ntrain, a.ntest
    t = {}
    X, t["cm"] = cpu_cm(batch)
    Xtr, Xte = X[:ntr], X[ntr:ntr + nte]
    rows = max(1, ntr // 16)
    t0 = time.perf_counter()
    kfn(Xtr, Xtr[:rows], a.sigma)
    t["kernel_train"] = (time.perf_counter() - t0) * (ntr / rows)
    t["kernel_test"], t["predict"] = cpu_test_side(Xtr, Xte, a, 16)
    nh = max(1, ntr // 2)
    Kh = kfn(Xtr[:nh], Xtr[:nh], a.sigma)
    Kh[np.diag_indices_from(Kh)] += a.lam
    t0 = time.perf_counter()
    c, info = lapack.dpotrf(Kh, lower=0, overwrite_a=1, clean=0)
    lapack.dpotrs(c, batch.labels[:nh], lower=0)
    t["cholesky"] = (time.perf_counter() - t0) * (ntr / nh) ** 3
    sample = ("all %d CMs; 1/16 of the rows of K_train (%dx%d) and K_test (%dx%d), scaled x16; "
              "dpotrf+dpotrs at N=%d scaled x%.0f (N^3); predict GEMV on the sampled rows x16"
              % (ntr + nte, ntr, ntr, ntr, nte, nh, (ntr / nh) ** 3))
    return sum(t.values()), t, sample


def run_reference(a):
    """The reference's CPU path on the host cores.  The two stages that hold ~95% of
    the time run once at full size: K_train (the oracle's OpenMP restatement of
    fgaussian_kernel, all N^2 entries as the reference computes them) and LAPACK
    dpotrf + dpotrs on K_train + lambda I at full N.  Each step then times the
    Coulomb matrices of every molecule and, on 1/16 of the test rows scaled by 16,
    K_test and the prediction GEMV.  value = the full-size stages + the mean step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import numpy as np
    from scipy.linalg import lapack

    from qml_gb300.synthetic import generate_molecules
    kfn = _kernel_fn(a.kernel)
    ntr, nte = a.ntrain, a.ntest
    batch = generate_molecules(ntr + nte, seed=a.seed)
    X, _ = cpu_cm(batch)
    Xtr, Xte = X[:ntr], X[ntr:ntr + nte]

    def step():
        _, t_cm = cpu_cm(batch)
        t_k, t_p = cpu_test_side(Xtr, Xte, a, 16)
        return {"cm": t_cm, "kernel_test": t_k, "predict": t_p}

    for _ in range(a.warmup):
        step()
    # the dominant stages at full size, once
    t0 = time.perf_counter()
    K = kfn(Xtr, Xtr, a.sigma)
    t_ktrain = time.perf_counter() - t0
    K[np.diag_indices_from(K)] += a.lam
    t0 = time.perf_counter()
    c, info = lapack.dpotrf(K, lower=0, overwrite_a=1, clean=0)
    lapack.dpotrs(c, batch.labels[:ntr], lower=0)
    t_chol = time.perf_counter() - t0
    del K, c
    steps = [step() for _ in range(a.steps)]
    parts = {k: statistics.mean(s[k] for s in steps) for k in steps[0]}
    parts["kernel_train"] = t_ktrain
    parts["cholesky"] = t_chol
    v = sum(parts.values())
    cores = os.cpu_count()
    sample = ("estimate: K_train (%dx%d) and dpotrf+dpotrs at N=%d timed once at full size; "
              "per step all %d CMs at full size, K_test and the predict GEMV on 1/16 of the "
              "%d test rows, scaled x16" % (ntr, ntr, ntr, ntr + nte, nte))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(a), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "estimate": True,
            "full_size_stages": ["kernel_train", "cholesky", "cm"],
            "scaled_stages": {"kernel_test": 16, "predict": 16},
            "dpotrf_info": int(info),
            "stages_s": parts}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------- GPU leg --

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _events(n):
    import torch
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def _span(e0, e1):
    return e0.elapsed_time(e1) / 1e3


def run_serving(a, dev):
    """Continuous-batching serving: one resident Gaussian model of serve_n molecules,
    Poisson query arrivals (1..4096 molecules, log-uniform), fits of N in
    [1000, 20000] interleaved every serve_fit_every-th arrival."""
    import torch

    from qml_gb300 import core, serving
    from qml_gb300.krr import KRR, molecules_to_device
    from qml_gb300.synthetic import generate_molecules

    pool = generate_molecules(a.serve_n + 30000, seed=a.seed + 7)
    train = pool.slice(0, a.serve_n)
    queries = pool.slice(a.serve_n, a.serve_n + 30000)
    z, r, o = molecules_to_device(train, device=dev)
    X = core.coulomb_matrix_batch(z, r, o, 23)
    y = torch.from_numpy(train.labels).to(dev)
    t0 = time.perf_counter()
    model = KRR(sigma=a.sigma, lam=a.lam, precision="mixed").fit(X, y)
    torch.cuda.synchronize()
    fit_s = time.perf_counter() - t0
    ex = serving.GpuExecutor(device=dev, n_streams=8)
    ex.add_model("main", X, model.alpha, a.sigma)
    # warm the streams (workspaces, pinned buffers) outside the measured run
    warm = serving.poisson_workload(50.0, 0.2, queries, "main", seed=a.seed + 1, max_query=4096)
    serving.Server(ex, serving.Scheduler(64 << 30, model_sizes={"main": a.serve_n})).run(warm)
    reqs = serving.poisson_workload(a.serve_rate, a.serve_seconds, queries, "main",
                                    fit_every=a.serve_fit_every, fit_sizes=(1000, 20000),
                                    seed=a.seed + 2, max_query=4096)
    sched = serving.Scheduler(budget_bytes=64 << 30, max_slots=8,
                              model_sizes={"main": a.serve_n})
    done = serving.Server(ex, sched).run(reqs)
    st = serving.latency_stats(done)
    fits = st.pop("fit_latency_ms")
    st.update({"resident_n": a.serve_n, "resident_fit_s": fit_s, "rate_hz": a.serve_rate,
               "duration_s": a.serve_seconds, "query_molecules": "log-uniform 1..4096",
               "fit_sizes": "log-uniform 1000..20000", "hbm_budget_gb": 64,
               "fit_latency_max_ms": max(fits) if fits else None})
    return st


def run_extra(a, dev, batch, X, stream):
    """Paths beside the KRR hot path, each timed on the GPU (CUDA events) and, where
    the CPU side is cheap, on the host: the other training kernel matrices, atomic
    Coulomb matrices, local kernels, the inverses and Bunch-Kaufman, the unsorted
    Coulomb matrix, XYZ file ingestion and model files."""
    import numpy as np
    import torch

    from oracle import oracle as orc
    from qml_gb300 import core
    from qml_gb300.krr import molecules_to_device
    ntr = a.ntrain
    out = {}

    def gpu_time(fn, reps=1):
        fn()
        torch.cuda.synchronize()
        e0, e1 = _events(2)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return _span(e0, e1) / reps

    Xtr = X[:ntr]

    def kernel(kind, emulated, **kw):
        return lambda: core.kernel_matrix(kind, Xtr, Xtr, a.sigma, symmetric=True,
                                          emulated=emulated, **kw)
    out["train_kernel_matrix_s"] = {
        "n": ntr,
        "gaussian_fp64": gpu_time(kernel("gaussian", False)),
        "gaussian_tensor": gpu_time(kernel("gaussian", True), reps=3),
        "laplacian_fp64": gpu_time(kernel("laplacian", False)),
        "laplacian_fixed": gpu_time(kernel("laplacian", True), reps=3),
        "linear_fp64": gpu_time(kernel("linear", False)),
        "linear_tensor": gpu_time(kernel("linear", True), reps=3),
        "matern_l2_order2_fp64": gpu_time(kernel("matern_l2", False, order=2)),
        "matern_l2_order2_tensor": gpu_time(kernel("matern_l2", True, order=2), reps=3),
        "sargan_2gammas_fp64": gpu_time(kernel("sargan", False, gammas=[1.0, 1.0 / 3.0])),
        "sargan_2gammas_fixed": gpu_time(kernel("sargan", True, gammas=[1.0, 1.0 / 3.0]), reps=3)}
    torch.cuda.empty_cache()

    sub = batch.slice(0, 25000)
    z, r, o = molecules_to_device(sub)
    t = gpu_time(lambda: core.atomic_coulomb_matrix_batch(z, r, o, 23, "row-norm"), reps=3)
    ns = 200
    c0 = time.perf_counter()
    for m in range(ns):
        orc.atomic_cm(*sub.molecule(m), None, 23, "row-norm")
    cpu = (time.perf_counter() - c0) * sub.n_mol / ns
    out["atomic_cm_rownorm"] = {"molecules": sub.n_mol, "atoms": int(sub.offsets[-1]),
                                "gpu_s": t, "cpu_oracle_s_scaled": cpu,
                                "cpu_sample": "%d molecules, 1 thread, scaled" % ns}
    nl = 2000
    sub = batch.slice(0, nl)
    zs, rs, os_ = molecules_to_device(sub)
    Xa = core.atomic_coulomb_matrix_batch(zs, rs, os_, 23, "row-norm")
    t = gpu_time(lambda: core.local_kernels("gaussian", Xa, Xa, os_, os_, [724.0], symmetric=True))
    te = gpu_time(lambda: core.local_kernels("gaussian", Xa, Xa, os_, os_, [724.0], symmetric=True,
                                             emulated=True))
    Xh = Xa.cpu().numpy()
    nh = np.diff(sub.offsets)
    rows = 50
    c0 = time.perf_counter()
    orc.local_kernels("gaussian", Xh[:int(sub.offsets[rows])], Xh, nh[:rows], nh, [724.0])
    cpu = (time.perf_counter() - c0) * nl / rows
    out["local_gaussian_kernel"] = {"molecules": nl, "gpu_s": t, "gpu_tensor_s": te,
                                    "cpu_oracle_s_scaled": cpu,
                                    "cpu_sample": "%d of %d rows, OpenMP on %d cores, scaled"
                                                  % (rows, nl, os.cpu_count())}
    # cho_invert, Bunch-Kaufman solve and inverse of an N=5000 Gaussian KRR matrix
    ni = 5000
    Xi = X[:ni]
    Ki = core.kernel_matrix("gaussian", Xi, Xi, 1000.0, symmetric=True, diag_shift=1e-4)
    tf = gpu_time(lambda: core.cho_invert(Ki, "fp64"))
    tm = gpu_time(lambda: core.cho_invert(Ki, "mixed"))
    yi = torch.ones(ni, dtype=torch.float64, device=dev)
    ts = gpu_time(lambda: core.bkf_solve(Ki, yi))
    tv = gpu_time(lambda: core.bkf_invert(Ki))
    Kh = np.asfortranarray(Ki.cpu().numpy())
    c0 = time.perf_counter()
    orc.cho_invert(Kh)
    ci = time.perf_counter() - c0
    c0 = time.perf_counter()
    orc.bkf_solve(Kh, np.ones(ni))
    cs = time.perf_counter() - c0
    c0 = time.perf_counter()
    orc.bkf_invert(Kh)
    cv = time.perf_counter() - c0
    # the same on a random symmetric indefinite matrix, where Bunch-Kaufman pivots
    # (2x2 pivots and interchanges at most steps)
    rng = np.random.default_rng(5000)
    Bh = rng.standard_normal((ni, ni))
    Sh = Bh + Bh.T
    Si = torch.from_numpy(Sh).to(dev)
    tsi = gpu_time(lambda: core.bkf_solve(Si, yi))
    tvi = gpu_time(lambda: core.bkf_invert(Si))
    Shf = np.asfortranarray(Sh)
    c0 = time.perf_counter()
    orc.bkf_solve(Shf, np.ones(ni))
    csi = time.perf_counter() - c0
    c0 = time.perf_counter()
    orc.bkf_invert(Shf)
    cvi = time.perf_counter() - c0
    out["inverses_n5000"] = {"cho_invert_gpu_fp64_s": tf, "cho_invert_gpu_mixed_s": tm,
                             "cho_invert_lapack_s": ci, "bkf_solve_gpu_s": ts,
                             "bkf_solve_lapack_s": cs, "bkf_invert_gpu_s": tv,
                             "bkf_invert_lapack_s": cv,
                             "indefinite": {"bkf_solve_gpu_s": tsi, "bkf_solve_lapack_s": csi,
                                            "bkf_invert_gpu_s": tvi, "bkf_invert_lapack_s": cvi,
                                            "matrix": "B + B^T, B standard normal, seed 5000"},
                             "cpu_sample": "scipy LAPACK, full size, OpenBLAS threads"}
    torch.cuda.empty_cache()

    # the other global kernels (GPU times in train_kernel_matrix_s) beside the OpenMP
    # oracle on a row sample of the same N x N matrix, scaled to all N rows
    Xg = X[:ntr].cpu().numpy()
    rows = 100
    g2 = [1.0, 1.0 / 3.0]
    samples = (("linear", lambda A: orc.linear_kernel(A, Xg)),
               ("matern_l2_order2", lambda A: orc.matern_kernel_l2(A, Xg, a.sigma, 2)),
               ("sargan_2gammas", lambda A: orc.sargan_kernel(A, Xg, a.sigma, g2)))
    other = {"n": ntr, "cpu_sample": "%d of %d rows, OpenMP on %d cores, scaled"
                                     % (rows, ntr, os.cpu_count())}
    for key, fn in samples:
        c0 = time.perf_counter()
        fn(Xg[:rows])
        other[key] = {"gpu_s": out["train_kernel_matrix_s"][key + "_fp64"],
                      "cpu_oracle_s_scaled": (time.perf_counter() - c0) * ntr / rows}
    other["linear"]["gpu_tensor_s"] = out["train_kernel_matrix_s"]["linear_tensor"]
    other["matern_l2_order2"]["gpu_tensor_s"] = out["train_kernel_matrix_s"]["matern_l2_order2_tensor"]
    other["sargan_2gammas"]["gpu_fixed_s"] = out["train_kernel_matrix_s"]["sargan_2gammas_fixed"]
    out["other_global_kernels"] = other
    del Xg

    # unsorted Coulomb matrices of the whole batch; the oracle is called once per
    # molecule, like the reference's per-molecule representation call
    zb, rb, ob = molecules_to_device(batch)
    t = gpu_time(lambda: core.coulomb_matrix_batch(zb, rb, ob, 23, "unsorted"), reps=3)
    ns = 2000
    c0 = time.perf_counter()
    for m in range(ns):
        orc.cm_unsorted(*batch.molecule(m), 23)
    cpu = (time.perf_counter() - c0) * batch.n_mol / ns
    out["unsorted_cm"] = {"molecules": batch.n_mol, "gpu_s": t, "cpu_oracle_s_scaled": cpu,
                          "cpu_sample": "%d molecules, 1 thread, scaled" % ns}
    del zb, rb, ob

    out["files"] = run_files(a, dev, batch, X)
    return out


def run_files(a, dev, batch, X):
    """The callers on either side of the path: XYZ files parsed into one ragged batch,
    copied to the device and turned into sorted Coulomb matrices; and a fitted model
    written to and read back from its .npz file. Wall-clock seconds on the host."""
    import shutil
    import tempfile

    import numpy as np
    import torch

    from qml_gb300 import core
    from qml_gb300 import io as qio
    from qml_gb300.krr import KRR
    from qml_gb300.representations import NUCLEAR_CHARGE
    symbol = {v: k for k, v in NUCLEAR_CHARGE.items()}
    nx = 5000
    tmp = tempfile.mkdtemp(prefix="qmlg_files_")
    try:
        paths = []
        for m in range(nx):
            z, r = batch.molecule(m)
            p = os.path.join(tmp, "%05d.xyz" % m)
            with open(p, "w") as f:
                f.write("%d\nsynthetic molecule %d\n" % (z.shape[0], m))
                for zi, ri in zip(z, r):
                    f.write("%s %.10f %.10f %.10f\n" % (symbol[int(zi)], ri[0], ri[1], ri[2]))
            paths.append(p)
        # one read_xyz per file, as a reference user builds one Compound per file
        c0 = time.perf_counter()
        for p in paths:
            qio.read_xyz(p)
        t_files = time.perf_counter() - c0
        c0 = time.perf_counter()
        qio.read_xyz_batch(paths, workers=1)
        t_serial = time.perf_counter() - c0
        c0 = time.perf_counter()
        parsed = qio.read_xyz_batch(paths)
        t_pool = time.perf_counter() - c0
        ref = batch.slice(0, nx)
        same = (np.array_equal(parsed.charges, ref.charges)
                and np.array_equal(parsed.offsets, ref.offsets)
                and float(np.max(np.abs(parsed.coordinates - ref.coordinates))) < 1e-9)

        def files_to_cm():
            z, r, o = qio.xyz_to_device(paths, dev)
            return core.coulomb_matrix_batch(z, r, o, 23)
        files_to_cm()
        torch.cuda.synchronize()
        c0 = time.perf_counter()
        files_to_cm()
        torch.cuda.synchronize()
        t_cm = time.perf_counter() - c0

        model = KRR(kernel=a.kernel, sigma=a.sigma, lam=a.lam)
        model.X = X[:a.ntrain]
        model.alpha = torch.linspace(-1.0, 1.0, a.ntrain, dtype=torch.float64, device=dev)
        mpath = os.path.join(tmp, "model.npz")
        c0 = time.perf_counter()
        qio.save_krr(mpath, model)
        t_save = time.perf_counter() - c0
        c0 = time.perf_counter()
        back = qio.load_krr(mpath, dev)
        torch.cuda.synchronize()
        t_load = time.perf_counter() - c0
        exact = bool(torch.equal(back.X, model.X) and torch.equal(back.alpha, model.alpha))
        return {"xyz": {"files": nx, "read_xyz_per_file_s": t_files,
                        "native_1_thread_s": t_serial, "native_all_threads_s": t_pool,
                        "threads": os.cpu_count(),
                        "files_to_device_cm_s": t_cm, "parsed_equal_to_source": bool(same)},
                "model_file": {"n_train": a.ntrain, "bytes": os.path.getsize(mpath),
                               "save_s": t_save, "load_to_device_s": t_load,
                               "round_trip_exact": exact}}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_batching(a, dev):
    """64 fits of uneven size (N log-uniform in [500, 8000]), each with its own
    sigma in {250, 500, 1000, 2000} and lambda in {1e-4, 1e-6, 1e-8}, recorded into
    one CUDA graph: the grouped path (one grouped launch per phase for all fits,
    autotuned tile parameters), beside the per-fit stream schedule in a graph and the
    same fits run one after another through the ordinary mixed solve."""
    import math

    import numpy as np
    import torch

    from qml_gb300 import core
    from qml_gb300.batch import BatchedKRR, Problem
    from qml_gb300.krr import KRR, molecules_to_device
    from qml_gb300.synthetic import generate_molecules

    rng = np.random.default_rng(a.seed + 11)
    pool = generate_molecules(16000, seed=a.seed + 12)
    z, r, o = molecules_to_device(pool, device=dev)
    Xall = core.coulomb_matrix_batch(z, r, o, 23)
    yall = torch.from_numpy(pool.labels).to(dev)
    probs = []
    for _ in range(a.batch_count):
        n = int(round(math.exp(rng.uniform(math.log(500), math.log(8000)))))
        start = int(rng.integers(0, 16000 - n + 1))
        probs.append(Problem(Xall[start:start + n].contiguous(), yall[start:start + n].contiguous(),
                             float(rng.choice([250.0, 500.0, 1000.0, 2000.0])),
                             float(rng.choice([1e-4, 1e-6, 1e-8]))))
    stream = torch.cuda.current_stream(dev)

    def replay_time(b, reps=3):
        b.capture()
        b.replay()
        torch.cuda.synchronize()
        e0, e1 = _events(2)
        e0.record(stream)
        for _ in range(reps):
            b.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        return _span(e0, e1) / reps

    # the grouped path (one grouped launch per phase), autotuned tile parameters
    b = BatchedKRR(probs, refine_steps=3)
    tuned = b.autotune(reps=1)
    graph_s = replay_time(b)
    alphas, reports = b.results()
    ok = sum(1 for rp in reports if rp["info"] == 0 and rp["flags"] == 0)
    lib = core.lib()
    torch.cuda.synchronize()
    c0 = lib.qmlg_launch_count()
    b.run_eager()
    grouped_launches = int(lib.qmlg_launch_count() - c0)
    del b
    torch.cuda.empty_cache()
    # the earlier schedule: each fit's own launches spread over 16 streams
    bs = BatchedKRR(probs, refine_steps=3, mode="streams", streams=16)
    streams_s = replay_time(bs)
    del bs
    torch.cuda.empty_cache()
    # the same fits one after another (kernel + mixed solve each, host-driven)
    t0 = time.perf_counter()
    for p in probs:
        KRR(sigma=p.sigma, lam=p.lam, precision="mixed").fit(p.X, p.y)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    sizes = [p.X.shape[0] for p in probs]
    return {"fits": len(probs), "n_min": min(sizes), "n_max": max(sizes),
            "n_sum": int(sum(sizes)), "graph_s": graph_s, "launches": grouped_launches,
            "streams_graph_s": streams_s, "sequential_s": seq_s,
            "speedup": seq_s / graph_s, "converged": ok,
            "tuned": {k: tuned[k] for k in ("tile_cols", "trsm_rows") if k in tuned}}


def run_large(a, dev, stream):
    """The 60000 train x 10000 test fits (Gaussian and Laplacian, sigma 1000, lambda
    1e-8, mixed), each timed twice after one warm-up (the median is reported)."""
    import torch

    from qml_gb300 import core
    from qml_gb300.krr import KRR, molecules_to_device
    from qml_gb300.synthetic import generate_molecules
    ntr, nte = a.large_train, a.large_test
    batch = generate_molecules(ntr + nte, seed=a.seed + 5)
    z, r, off = molecules_to_device(batch, device=dev)
    y = torch.from_numpy(batch.labels).to(dev)
    out = {"n_train": ntr, "n_test": nte, "sigma": a.sigma, "lambda": a.lam}
    for kind in ("gaussian", "laplacian"):
        times, rep = [], None
        for k in range(3):
            torch.cuda.synchronize()
            e = _events(5)
            e[0].record(stream)
            X = core.coulomb_matrix_batch(z, r, off, 23)
            e[1].record(stream)
            K = core.kernel_matrix(kind, X[:ntr], X[:ntr], a.sigma, symmetric=True, emulated=True)
            e[2].record(stream)
            alpha, rep = core.solve(K, y[:ntr], a.lam, precision="mixed")
            e[3].record(stream)
            core.predict(kind, X[:ntr], X[ntr:ntr + nte], a.sigma, alpha, emulated=True)
            e[4].record(stream)
            torch.cuda.synchronize()
            del K
            if k > 0:
                times.append([_span(e[0], e[4]), _span(e[1], e[2]), _span(e[2], e[3]),
                              _span(e[3], e[4])])
        times.sort()
        med = times[len(times) // 2]
        out[kind] = {"fit_predict_s": med[0], "kernel_s": med[1], "solve_s": med[2],
                     "predict_s": med[3], "refine_steps": rep["outer_iterations"],
                     "fell_back": rep["fell_back"]}
        torch.cuda.empty_cache()
    return out


def run_ours(a):
    import torch
    import torch.distributed as dist

    from qml_gb300 import core, replicas
    from qml_gb300.krr import KRR, molecules_to_device
    from qml_gb300.synthetic import generate_molecules

    world, rank, local = replicas.rank_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    ntr, nte = a.ntrain, a.ntest
    batch = generate_molecules(ntr + nte, seed=replicas.replica_seed(a.seed, rank))
    z, r, off = molecules_to_device(batch, device=dev)
    y = torch.from_numpy(batch.labels).to(dev)
    stream = torch.cuda.current_stream(dev)

    def step(precision="mixed"):
        X = core.coulomb_matrix_batch(z, r, off, 23)
        model = KRR(kernel=a.kernel, sigma=a.sigma, lam=a.lam, precision=precision)
        model.fit(X[:ntr], y[:ntr])
        return model.predict(X[ntr:ntr + nte]), model

    for _ in range(a.warmup):
        step()
    barrier()
    with ClockSampler(local) as clocks:
        ev0, ev1 = _events(2)
        ev0.record(stream)
        for _ in range(a.steps):
            yhat, model = step()
        ev1.record(stream)
        barrier()
    ms = replicas.max_over_ranks(ev0.elapsed_time(ev1) / a.steps, device=dev)
    report = model.report
    del model, yhat

    # end to end through the public API with host buffers (pinned), copies inside
    hz = torch.from_numpy(batch.charges).pin_memory()
    hr = torch.from_numpy(batch.coordinates).pin_memory()
    ho = torch.from_numpy(batch.offsets).pin_memory()
    hy = torch.from_numpy(batch.labels[:ntr].copy()).pin_memory()
    hout = torch.empty(nte, dtype=torch.float64).pin_memory()
    h2d = hz.numel() * 8 + hr.numel() * 8 + ho.numel() * 8 + hy.numel() * 8
    d2h = nte * 8

    def e2e_step():
        dz, dr, do, dy = (t.to(dev, non_blocking=True) for t in (hz, hr, ho, hy))
        X = core.coulomb_matrix_batch(dz, dr, do, 23)
        m = KRR(kernel=a.kernel, sigma=a.sigma, lam=a.lam, precision="mixed").fit(X[:ntr], dy)
        hout.copy_(m.predict(X[ntr:ntr + nte]), non_blocking=True)

    e2e_step()
    barrier()
    e0, e1 = _events(2)
    e0.record(stream)
    for _ in range(a.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_s = replicas.max_over_ranks(_span(e0, e1) / a.steps, device=dev)

    # per-stage times of one mixed step (events between stages), and the mixed
    # factorisation alone on a copy of the same K
    evs = _events(5)
    evs[0].record(stream)
    X = core.coulomb_matrix_batch(z, r, off, 23)
    evs[1].record(stream)
    K = core.kernel_matrix(a.kernel, X[:ntr], X[:ntr], a.sigma, symmetric=True, emulated=True)
    evs[2].record(stream)
    Kf = K.clone()  # for the factorisation timed alone below (outside the stages)
    c0 = torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    alpha, rep = core.solve(K, y[:ntr], a.lam, precision="mixed")
    evs[3].record(stream)
    core.predict(a.kernel, X[:ntr], X[ntr:ntr + nte], a.sigma, alpha, emulated=True)
    evs[4].record(stream)
    torch.cuda.synchronize()
    stages = {name: _span(evs[k], evs[k + 1])
              for k, name in enumerate(["cm", "kernel_train", "solve", "predict"])}
    stages["solve"] = _span(c0, evs[3])
    f0, f1 = _events(2)
    f0.record(stream)
    core.cholesky(Kf, a.lam, precision="mixed")
    f1.record(stream)
    torch.cuda.synchronize()
    stages["factor"] = _span(f0, f1)
    del K, Kf

    # dominant kernel: the emulated trailing update of the mixed Cholesky
    # (first outer step of this workload: C (n-512)^2 lower, P (n-512) x 512)
    nsy, ksy = ntr - 512, 512
    Csy = torch.rand((nsy, nsy), dtype=torch.float64, device=dev)
    Psy = torch.rand((nsy, ksy), dtype=torch.float64, device=dev)
    core.syrk_emulated(Csy, Psy)
    k0, k1 = _events(2)
    nk = 3
    k0.record(stream)
    for _ in range(nk):
        core.syrk_emulated(Csy, Psy)
    k1.record(stream)
    torch.cuda.synchronize()
    syrk_s = _span(k0, k1) / nk
    del Csy, Psy
    torch.cuda.empty_cache()

    # the plain FP64 GPU path: fit + predict timed --fp64-reps times; the first
    # repeat's alpha (FP64 factor + refinement) is compared with the mixed solve of
    # the identical FP64 K
    fp64 = {}
    if a.fp64_reps > 0:
        times, err, rep_f = [], None, None
        for k in range(a.fp64_reps):
            e = _events(5)
            e[0].record(stream)
            X = core.coulomb_matrix_batch(z, r, off, 23)
            K64 = core.kernel_matrix(a.kernel, X[:ntr], X[:ntr], a.sigma, symmetric=True)
            e[1].record(stream)
            Kc = K64.clone() if k == 0 else None
            e[2].record(stream)
            alpha_f, rep_f = core.solve(K64, y[:ntr], a.lam, precision="fp64")
            core.predict(a.kernel, X[:ntr], X[ntr:ntr + nte], a.sigma, alpha_f)
            e[3].record(stream)
            torch.cuda.synchronize()
            times.append(_span(e[0], e[1]) + _span(e[2], e[3]))
            del K64
            if k == 0:
                alpha_m, rep_m = core.solve(Kc, y[:ntr], a.lam, precision="mixed")
                err = float(torch.linalg.norm(alpha_m - alpha_f) / torch.linalg.norm(alpha_f))
                del Kc
            torch.cuda.empty_cache()
        med = statistics.median(times)
        fp64 = {"fit_predict_s_median": med, "fit_predict_s": times,
                "speedup_mixed_vs_fp64": med / (ms / 1e3),
                "alpha_rel_err_mixed_vs_fp64_refined": err,
                "fp64_refine_steps": rep_f["outer_iterations"]}

    # our kernel launches per step, counted by the library itself
    lib = core.lib()
    torch.cuda.synchronize()
    c0 = lib.qmlg_launch_count()
    step()
    torch.cuda.synchronize()
    launches = int(lib.qmlg_launch_count() - c0) * a.steps

    large = run_large(a, dev, stream) if not a.no_large and rank == 0 else None
    serving_stats = run_serving(a, dev) if not a.no_serving else None
    batching_stats = run_batching(a, dev) if not a.no_batching else None
    extra = None
    if not a.no_extra and rank == 0:
        X = core.coulomb_matrix_batch(z, r, off, 23)
        extra = run_extra(a, dev, batch, X, stream)

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    # roofline of the dominant kernel (the emulated trailing update): 36 bf16
    # digit-plane products of the lower triangle, 36 n(n+1) k flops per launch; the
    # FP64-equivalent rate (n(n+1) k flops) beside it; and the whole mixed
    # factorisation's digit-plane rate, 36 N^3 / 3 flops over its measured time
    flops = 36.0 * nsy * (nsy + 1) * ksy
    achieved = flops / syrk_s / 1e12
    fact_tflops = 36.0 * ntr ** 3 / 3.0 / stages["factor"] / 1e12
    roofline = {"kernel": "emu_tc_kernel<syrk> (C %dx%d lower -= P P^T, k=%d, 8 digit planes)"
                % (nsy, nsy, ksy),
                "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak,
                # DRAM bytes per launch: 0.7305e9 read+written by one ncu capture of
                # the same kernel at n = 8192, k = 512, scaled by the lower-triangle size
                "traffic": 0.7305e9 * (nsy / 8192.0) ** 2,
                "traffic_note": "scaled from an ncu capture at n=8192, k=512",
                "algorithmic_bytes": 8.0 * nsy * (nsy + 1) + 8.0 * nsy * ksy + 16.0 * nsy * ksy,
                "peak_source": "measured bf16 (MEASURED_PEAKS.json)" if peaks else "fallback",
                "launch_s": syrk_s,
                "fp64_equivalent_tflops": nsy * (nsy + 1) * ksy / syrk_s / 1e12,
                "factorisation_tflops": fact_tflops, "factorisation_frac": fact_tflops / peak}
    cpu = None
    if not a.no_cpu:
        total, parts, sample = cpu_baseline_sample(batch, a)
        cpu = {"value": total, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": sample, "stages_s": parts}
    headline = {"fit_predict_s": ms / 1e3, "e2e_s": e2e_s,
                "fp64_fit_predict_s": fp64.get("fit_predict_s_median"),
                "speedup_mixed_vs_fp64": fp64.get("speedup_mixed_vs_fp64"),
                "alpha_rel_err_vs_fp64_refined": fp64.get("alpha_rel_err_mixed_vs_fp64_refined"),
                "refine_steps": report.get("outer_iterations"),
                "fell_back": report.get("fell_back")}
    if serving_stats:
        headline.update({"serving_p50_ms": serving_stats["p50_ms"],
                         "serving_p99_ms": serving_stats["p99_ms"],
                         "serving_molecules_per_s": serving_stats["molecules_per_s"]})
    if large:
        headline.update({"fit60000_gaussian_s": large["gaussian"]["fit_predict_s"],
                         "fit60000_laplacian_s": large["laplacian"]["fit_predict_s"]})
    if batching_stats:
        headline["batch64_graph_s"] = batching_stats["graph_s"]
    line = {"metric": METRIC, "value": ms / 1e3, "unit": UNIT,
            "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(a),
            "e2e": {"value": e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clocks.summary(), "roofline": roofline,
            "cpu_baseline": cpu,
            "fits_per_s": replicas.job_throughput(1.0, ms / 1e3, world),
            "other_paths": extra, "batching": batching_stats, "large": large,
            "serving": serving_stats, "stages_s": stages, "solve_report": report,
            "fp64_path": fp64,
            "headline": headline}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
