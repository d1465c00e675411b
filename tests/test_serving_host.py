"""Serving scheduler and loop on the host (no GPU): admission against the HBM
budget, merging of predictions, fits one at a time, latency accounting."""
import threading

import numpy as np

from qml_gb300 import serving
from qml_gb300.serving import (Request, Scheduler, Server, fit_bytes, merge_molecules,
                                predict_bytes, resident_bytes)
from qml_gb300.synthetic import generate_molecules


def mk(rid, kind, model, n, t, seed=None):
    b = generate_molecules(n, seed=rid if seed is None else seed)
    return Request(rid, kind, model, b.charges, b.coordinates, b.offsets, t,
                   labels=b.labels if kind == "fit" else None)


def test_merge_molecules_offsets():
    reqs = [mk(0, "predict", "m", 3, 0.0), mk(1, "predict", "m", 5, 0.0)]
    z, r, off, ranges = merge_molecules(reqs)
    assert ranges == [(0, 3), (3, 8)]
    assert off.shape == (9,) and off[0] == 0 and off[-1] == z.shape[0] == r.shape[0]
    assert np.array_equal(off[3:] - off[3], reqs[1].offsets)


def test_predictions_merge_and_respect_slots():
    s = Scheduler(budget_bytes=1 << 40, max_slots=2, max_batch_molecules=10,
                  model_sizes={"m": 1000, "k": 1000})
    for i, (model, n) in enumerate([("m", 4), ("k", 3), ("m", 5), ("m", 4)]):
        s.submit(mk(i, "predict", model, n, 0.0))
    b1 = s.next_batch()
    assert [r.rid for r in b1] == [0, 2]          # same model, up to 10 molecules
    b2 = s.next_batch()
    assert [r.rid for r in b2] == [1]
    assert s.next_batch() is None                  # both slots taken
    s.release(b1)
    assert [r.rid for r in s.next_batch()] == [3]


def test_budget_admission_and_rejection():
    s = Scheduler(budget_bytes=fit_bytes(2000) + predict_bytes(10, 1000) + resident_bytes(1000),
                  max_slots=4, model_sizes={"m": 1000})
    assert s.in_use == resident_bytes(1000)
    s.submit(mk(0, "fit", "f", 2000, 0.0))
    s.submit(mk(1, "fit", "g", 1500, 0.0))
    s.submit(mk(2, "predict", "m", 10, 0.0))
    first = s.next_batch()
    assert first[0].rid == 0 and s.fit_running
    second = s.next_batch()                        # second fit waits; the query proceeds
    assert second[0].rid == 2
    assert s.next_batch() is None
    s.release(first)
    assert s.model_sizes["f"] == 2000
    assert s.next_batch()[0].rid == 1
    big = Scheduler(budget_bytes=1 << 20, model_sizes={"m": 1000})
    big.submit(mk(5, "fit", "h", 3000, 0.0))
    rej = big.next_batch()
    assert rej[0].error is not None


def test_queries_wait_for_their_model():
    s = Scheduler(budget_bytes=1 << 40, model_sizes={})
    s.submit(mk(0, "predict", "f", 3, 0.0))
    s.submit(mk(1, "fit", "f", 500, 0.0))
    b = s.next_batch()
    assert b[0].kind == "fit"
    assert s.next_batch() is None
    s.release(b)
    assert s.next_batch()[0].rid == 0


class FakeEvent:
    def __init__(self, ready_at, clock):
        self.ready_at, self.clock = ready_at, clock

    def query(self):
        return self.clock() >= self.ready_at


class FakeExecutor:
    """Completes each prediction batch after a fixed delay; results are per-molecule
    functions of the molecule alone, so merging cannot change them."""

    def __init__(self, clock, delay=0.002):
        self.clock, self.delay, self.batches = clock, delay, []

    def launch_predict(self, batch):
        self.batches.append([r.rid for r in batch])
        ev = FakeEvent(self.clock() + self.delay, self.clock)

        def finish():
            for r in batch:
                r.result = np.array([float(np.sum(r.charges[r.offsets[m]:r.offsets[m + 1]]))
                                     for m in range(r.n_mol)])
        return ev, finish

    def run_fit(self, req):
        req.result = np.zeros(1)


def test_server_loop_with_fake_executor():
    import time
    clock = time.perf_counter
    ex = FakeExecutor(clock)
    sched = Scheduler(budget_bytes=1 << 40, max_slots=2, model_sizes={"m": 100})
    arrivals = [mk(i, "predict", "m", 1 + (i % 7), 0.0005 * i) for i in range(40)]
    arrivals.append(mk(40, "fit", "f", 50, 0.001))
    done = Server(ex, sched, clock=clock).run(arrivals)
    assert len(done) == 41
    assert all(r.result is not None for r in done)
    assert all(r.done >= r.arrival for r in done)
    assert any(len(b) > 1 for b in ex.batches)     # some predictions were merged
    stats = serving.latency_stats(done)
    assert stats["queries"] == 40 and stats["fits"] == 1 and stats["p99_ms"] >= stats["p50_ms"]
    alone = mk(3, "predict", "m", 1 + 3, 0.0)
    ex.launch_predict([alone])[1]()
    mixed = next(r for r in done if r.rid == 3)
    assert np.array_equal(alone.result, mixed.result)


def test_poisson_workload_shape():
    pool = generate_molecules(500, seed=3)
    reqs = serving.poisson_workload(200.0, 0.5, pool, "m", fit_every=10, fit_sizes=(100, 200),
                                    seed=1, max_query=64)
    assert 50 < len(reqs) < 200
    assert all(1 <= r.n_mol <= 64 for r in reqs if r.kind == "predict")
    assert sum(r.kind == "fit" for r in reqs) >= 5
    assert all(reqs[i].arrival <= reqs[i + 1].arrival for i in range(len(reqs) - 1))


def test_costs_follow_the_library_workspace_sizes():
    from qml_gb300 import _lib
    lib = _lib.load()
    n = 3000
    ws = max(lib.qmlg_gaussian_kernel_emulated_workspace_size(n, n, 276, 1),
             lib.qmlg_solve_workspace_size(n, 1))
    assert fit_bytes(n) >= 8 * n * n + ws
    assert fit_bytes(n, "laplacian") >= 8 * n * n + lib.qmlg_solve_workspace_size(n, 1)
    assert predict_bytes(100, n) >= lib.qmlg_predict_emulated_workspace_size(n, 100, 276)
    assert predict_bytes(100, n, "laplacian") >= \
        lib.qmlg_predict_laplacian_fixed_workspace_size(n, 100, 276)
    # grows with the problem
    assert fit_bytes(2 * n) > fit_bytes(n) and predict_bytes(200, n) > predict_bytes(100, n)


def test_fitted_models_stay_accounted():
    s = Scheduler(budget_bytes=1 << 40, model_sizes={})
    s.submit(mk(0, "fit", "f", 300, 0.0))
    b = s.next_batch()
    assert s.in_use == fit_bytes(300)
    s.release(b)
    assert s.in_use == resident_bytes(300) and s.model_sizes["f"] == 300


def test_failed_fit_answers_its_waiting_queries():
    # a fit that fails on the GPU (here: an allocation failure although the budget
    # admitted it) releases its cost; the queries for its model get the fit's error
    s = Scheduler(budget_bytes=1 << 40, model_sizes={"m": 100})
    s.submit(mk(0, "fit", "f", 200, 0.0))
    s.submit(mk(1, "predict", "f", 3, 0.0))
    s.submit(mk(2, "predict", "m", 2, 0.0))
    fit = s.next_batch()
    assert fit[0].rid == 0
    fit[0].error = "RuntimeError('CUDA out of memory')"
    s.release(fit)
    assert s.in_use == resident_bytes(100) and "f" not in s.model_sizes
    out = [s.next_batch(), s.next_batch()]
    rej = next(b for b in out if b[0].rid == 1)
    assert rej[0].error is not None and "failed to fit" in rej[0].error
    ok = next(b for b in out if b[0].rid == 2)
    assert ok[0].error is None


class FailingFitExecutor(FakeExecutor):
    """A fake whose fits of one model raise the error an allocation failure raises."""

    def run_fit(self, req):
        if req.model == "bad":
            raise RuntimeError("CUDA out of memory. Tried to allocate 3.20 GiB")
        req.result = np.zeros(1)


def test_server_survives_a_fit_that_fails_to_allocate():
    import time
    clock = time.perf_counter
    ex = FailingFitExecutor(clock)
    sched = Scheduler(budget_bytes=1 << 40, max_slots=2, model_sizes={"m": 100})
    arrivals = [mk(0, "fit", "bad", 60, 0.0), mk(1, "predict", "bad", 2, 0.0005),
                mk(2, "predict", "m", 3, 0.001), mk(3, "fit", "good", 40, 0.0015),
                mk(4, "predict", "good", 2, 0.002), mk(5, "predict", "bad", 1, 0.003)]
    done = Server(ex, sched, clock=clock).run(arrivals)
    assert len(done) == 6
    by = {r.rid: r for r in done}
    assert "out of memory" in by[0].error
    assert by[1].error is not None and by[5].error is not None
    assert by[2].error is None and by[3].error is None and by[4].error is None
    assert by[4].result is not None
    # everything admitted was released; the two fitted models stay accounted
    assert sched.in_use == resident_bytes(100) + resident_bytes(40)
    assert sched.slots == 0 and not sched.fit_running


class FailingLaunchExecutor(FakeExecutor):
    """A fake whose prediction launches for one model raise (as an allocation that
    fails would), and whose result copy for another model raises."""

    def launch_predict(self, batch):
        if batch[0].model == "oom":
            raise RuntimeError("CUDA out of memory. Tried to allocate 1.00 GiB")
        ev, finish = super().launch_predict(batch)
        if batch[0].model == "bad_copy":
            def fail():
                raise RuntimeError("copy failed")
            return ev, fail
        return ev, finish


def test_server_survives_failed_prediction_launches():
    import time
    clock = time.perf_counter
    ex = FailingLaunchExecutor(clock)
    sched = Scheduler(budget_bytes=1 << 40, max_slots=2,
                      model_sizes={"m": 100, "oom": 100, "bad_copy": 100})
    arrivals = [mk(0, "predict", "oom", 3, 0.0), mk(1, "predict", "m", 2, 0.0005),
                mk(2, "predict", "bad_copy", 4, 0.001), mk(3, "predict", "m", 1, 0.0015)]
    done = Server(ex, sched, clock=clock).run(arrivals)
    by = {r.rid: r for r in done}
    assert len(done) == 4
    assert "out of memory" in by[0].error and "copy failed" in by[2].error
    assert by[1].error is None and by[3].error is None and by[1].result is not None
    # every admitted cost and slot was released
    assert sched.slots == 0 and sched.in_use == 3 * resident_bytes(100)
