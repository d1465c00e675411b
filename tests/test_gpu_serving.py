"""Serving on the GPU: a resident model, Poisson queries mixed with a fit; each
query's result is the same alone and in the mix (within the kernel's 1e-12 bound)
and matches the oracle prediction."""
import numpy as np
import pytest
import torch

from qml_gb300 import core, serving
from qml_gb300.krr import KRR, molecules_to_device
from qml_gb300.synthetic import generate_molecules

pytestmark = pytest.mark.gpu


def test_serving_mix_equals_alone(cuda, oracle):
    ntr = 3000
    train = generate_molecules(ntr, seed=101)
    z, r, o = molecules_to_device(train)
    X = core.coulomb_matrix_batch(z, r, o, 23)
    y = torch.from_numpy(train.labels).to(cuda)
    model = KRR(sigma=1000.0, lam=1e-8, precision="mixed").fit(X, y)
    ex = serving.GpuExecutor(n_streams=3)
    ex.add_model("main", X, model.alpha, 1000.0)
    pool = generate_molecules(4000, seed=102)
    reqs = serving.poisson_workload(400.0, 0.5, pool, "main", fit_every=40, fit_sizes=(500, 1500),
                                    seed=5, max_query=512)
    sched = serving.Scheduler(budget_bytes=8 << 30, max_slots=3,
                              model_sizes={"main": ntr})
    done = serving.Server(ex, sched).run(reqs)
    assert len(done) == len(reqs)
    assert all(r.error is None for r in done)
    stats = serving.latency_stats(done)
    assert stats["queries"] > 50 and stats["fits"] >= 1
    Xo = oracle.cm_sorted_batch(train.charges, train.coordinates, train.offsets, 23)
    alpha = model.alpha.cpu().numpy()
    preds = [r for r in done if r.kind == "predict"]
    assert all(r.path == "tensor" and r.flag == 0 for r in preds), \
        sorted({(r.path, r.flag) for r in preds})
    for req in preds[:12]:
        # alone: the same request as its own batch through the same executor
        alone = serving.Request(-1, "predict", "main", req.charges, req.coordinates, req.offsets, 0.0)
        ev, finish = ex.launch_predict([alone])
        ev.synchronize()
        finish()
        # the result depends on the request's own molecules only: bit for bit here
        assert np.array_equal(alone.result, req.result)
        # against the oracle: each kernel entry is within 1e-12 relative, so the
        # prediction is within 1e-12 of sum_j |k_ij alpha_j| (alpha is large and
        # cancels: |alpha| reaches ~1e8 at lambda = 1e-8)
        Xq = oracle.cm_sorted_batch(req.charges, req.coordinates, req.offsets, 23)
        Ks = oracle.gaussian_kernel(Xo, Xq, 1000.0)
        expect = Ks.T @ alpha
        scale = np.abs(Ks.T) @ np.abs(alpha)
        assert np.max(np.abs(req.result - expect) / scale) <= 1e-12


def test_serving_laplacian_model_mix_equals_alone(cuda, oracle):
    # a Laplacian model (the reference's end-to-end KRR test uses the Laplacian
    # kernel, sigma = 10^4.2, lambda = 1e-10: tests/test_energy_krr_cmat.py:97-113):
    # queries take the fixed-point fused prediction, fits in the mix create
    # Laplacian models too, and each query's result is the same alone and in the mix
    sigma, lam, ntr = 10 ** 4.2, 1e-10, 3000
    train = generate_molecules(ntr, seed=111)
    z, r, o = molecules_to_device(train)
    X = core.coulomb_matrix_batch(z, r, o, 23)
    y = torch.from_numpy(train.labels).to(cuda)
    model = KRR(kernel="laplacian", sigma=sigma, lam=lam, precision="mixed").fit(X, y)
    ex = serving.GpuExecutor(n_streams=3)
    ex.add_model("lap", X, model.alpha, sigma, kernel="laplacian")
    pool = generate_molecules(4000, seed=112)
    reqs = serving.poisson_workload(400.0, 0.5, pool, "lap", fit_every=40, fit_sizes=(500, 1500),
                                    seed=6, max_query=512, fit_kernel="laplacian", fit_sigma=sigma)
    sched = serving.Scheduler(budget_bytes=8 << 30, max_slots=3, model_sizes={"lap": ntr},
                              model_kinds={"lap": "laplacian"})
    done = serving.Server(ex, sched).run(reqs)
    assert len(done) == len(reqs) and all(r.error is None for r in done)
    fits = [r for r in done if r.kind == "fit"]
    assert fits and all(ex.models[r.model][3] == "laplacian" for r in fits)
    preds = [r for r in done if r.kind == "predict"]
    assert len(preds) > 50
    assert all(r.path == "fixed" and r.flag == 0 for r in preds), \
        sorted({(r.path, r.flag) for r in preds})
    Xo = oracle.cm_sorted_batch(train.charges, train.coordinates, train.offsets, 23)
    alpha = model.alpha.cpu().numpy()
    for req in preds[:12]:
        alone = serving.Request(-1, "predict", "lap", req.charges, req.coordinates, req.offsets, 0.0)
        ev, finish = ex.launch_predict([alone])
        ev.synchronize()
        finish()
        assert np.array_equal(alone.result, req.result)
        Xq = oracle.cm_sorted_batch(req.charges, req.coordinates, req.offsets, 23)
        Ks = oracle.laplacian_kernel(Xo, Xq, sigma)
        scale = np.abs(Ks.T) @ np.abs(alpha)
        assert np.max(np.abs(req.result - Ks.T @ alpha) / scale) <= 1e-12


@pytest.mark.parametrize("kernel", ["gaussian", "laplacian"])
def test_admission_costs_cover_the_allocator_peak(cuda, kernel):
    # the scheduler admits work by fit_bytes / predict_bytes; the device memory a
    # fit and a merged prediction really take (the caching allocator's peak above
    # what was held before) must stay under those costs, and the costs may not
    # overstate it by more than the per-molecule allowance and the rounding slack
    ntr, nq = 3000, 700
    ex = serving.GpuExecutor(n_streams=1)
    torch.cuda.synchronize()
    train = generate_molecules(ntr, seed=201)
    req = serving.Request(0, "fit", "m", train.charges, train.coordinates, train.offsets, 0.0,
                          labels=train.labels, kernel=kernel)
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    try:
        ex.run_fit(req)
    finally:
        core.lib().qmlg_set_thread_sm_limit(0)
    torch.cuda.synchronize()
    peak = torch.cuda.max_memory_allocated() - base
    cost = serving.fit_bytes(ntr, kernel)
    assert peak <= cost, (peak, cost)
    assert cost - peak <= serving._ALLOC_SLACK + serving._MOL_BYTES * ntr, (peak, cost)
    # what stays is the model: its Coulomb matrices and alpha (the workspace cache
    # of the fit stream stays too, owned by the process, not by the model)
    X, alpha, _, _ = ex.models["m"]
    assert X.numel() * 8 + alpha.numel() * 8 == serving.resident_bytes(ntr)

    q = generate_molecules(nq, seed=202)
    qreq = serving.Request(1, "predict", "m", q.charges, q.coordinates, q.offsets, 0.0)
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    ev, finish = ex.launch_predict([qreq])
    ev.synchronize()
    peak = torch.cuda.max_memory_allocated() - base
    finish()
    cost = serving.predict_bytes(nq, ntr, kernel)
    assert peak <= cost, (peak, cost)
    assert cost - peak <= serving._ALLOC_SLACK + serving._MOL_BYTES * nq, (peak, cost)
    assert qreq.result.shape == (nq,) and np.all(np.isfinite(qreq.result))
