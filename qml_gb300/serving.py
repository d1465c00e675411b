"""Continuous-batching KRR serving on one GPU.

Resident models are the training Coulomb matrices and their alpha, both kept in HBM.
Requests arrive over time:
  * predict: a batch of molecules against a named model;
  * fit: molecules + labels -> a new resident model.

The scheduler runs one host loop.  On every turn it does three things:
  * it moves arrived requests into the queue;
  * it retires finished work (CUDA events polled, never waited on);
  * it admits queued requests while slots are free and the HBM budget allows.

Admitted predictions of the same model are merged into one launch.  The merged
launch is one Coulomb-matrix kernel and one fused prediction (tensor cores for a
Gaussian model, fixed-point L1 sums for a Laplacian one), and the results are split
back per request.  It runs on one of several CUDA streams, so
it overlaps with other batches and with fits.  Fits synchronise internally (the
solve takes refinement decisions on the host), so they run on a worker thread
with their own stream.  The host loop keeps admitting predictions meanwhile.

Each prediction depends only on its own molecules.  The per-tile partial sums are
reduced in a fixed order, and every row is scaled independently.  So a request's
result is the same alone and in a mix, up to the kernel's 1e-12 bound: the
digit-plane count may differ when a batch's value range changes.
"""
from __future__ import annotations

import collections
import math
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional

import numpy as np

CM_SIZE = 23
FEATURES = CM_SIZE * (CM_SIZE + 1) // 2


@dataclass
class Request:
    rid: int
    kind: str                    # "predict" | "fit"
    model: str                   # model to query, or name of the model a fit creates
    charges: np.ndarray
    coordinates: np.ndarray
    offsets: np.ndarray
    arrival: float               # seconds on the server clock
    labels: Optional[np.ndarray] = None
    sigma: float = 1000.0
    lam: float = 1e-8
    admitted: float = math.nan
    done: float = math.nan
    result: Optional[np.ndarray] = None
    error: Optional[str] = None
    path: str = ""               # "tensor" / "fixed", or "fp64" when the fast path's bound failed
    flag: int = 0
    kernel: str = "gaussian"     # fit requests: the kernel of the model they create

    @property
    def n_mol(self) -> int:
        return int(self.offsets.shape[0] - 1)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


# Per-molecule device bytes of a request's own tensors: charges and coordinates of
# up to CM_SIZE atoms (4 doubles each), the offset, the label or output, and the
# Coulomb-matrix row.
_MOL_BYTES = CM_SIZE * 4 * 8 + 8 + 8 + FEATURES * 8
# torch's caching allocator rounds every block up (large ones to 2 MiB); a request
# makes fewer than eight device allocations
_ALLOC_SLACK = 16 << 20


def _workspace(name: str, *args) -> int:
    """A workspace size from the library (pure host arithmetic, no GPU needed)."""
    from . import _lib
    return int(getattr(_lib.load(), name)(*args))


def fit_bytes(n: int, kernel: str = "gaussian") -> int:
    """HBM a fit holds while it runs: its molecules and Coulomb matrices, K (8 n^2),
    alpha, and the one workspace the kernel matrix and the mixed solve share (the
    library's own sizes: digit planes, block inverses, residual partials)."""
    if kernel == "laplacian":
        kws = _workspace("qmlg_laplacian_kernel_fixed_workspace_size", n, n, FEATURES, 1)
    else:
        kws = _workspace("qmlg_gaussian_kernel_emulated_workspace_size", n, n, FEATURES, 1)
    sws = _workspace("qmlg_solve_workspace_size", n, 1)
    return 8 * n * n + (_MOL_BYTES + 8) * n + max(kws, sws) + _ALLOC_SLACK


def resident_bytes(n: int) -> int:
    """HBM a fitted model keeps: its training Coulomb matrices and alpha."""
    return (FEATURES + 1) * 8 * n


def predict_bytes(n_query: int, n_train: int, kernel: str = "gaussian") -> int:
    """HBM a merged prediction batch holds: its molecules, Coulomb matrices and
    outputs, and the fused prediction's workspace (the library's own size: digit
    planes of both sides and partial sums for a Gaussian model, fixed-point
    features and partial sums for a Laplacian one)."""
    if kernel == "laplacian":
        ws = _workspace("qmlg_predict_laplacian_fixed_workspace_size", n_train, n_query, FEATURES)
    else:
        ws = _workspace("qmlg_predict_emulated_workspace_size", n_train, n_query, FEATURES)
    return _MOL_BYTES * n_query + ws + _ALLOC_SLACK


class Scheduler:
    """Host-side admission and batching (no GPU).  `budget_bytes` caps the HBM that
    resident models and admitted work may hold together; `max_slots` caps concurrent
    prediction batches; `max_batch_molecules` caps one merged prediction launch.

    The costs are the library's workspace sizes plus each request's own tensors
    (fit_bytes, predict_bytes, resident_bytes); a GPU test checks them against the
    allocator's peak.  The per-stream workspace cache (core.workspaces) keeps the
    largest workspace each stream has used, so the process holds that much more than
    the admitted costs between requests.  A fit that fails (an allocation that fails
    although the budget allowed it, for example) releases its cost, and the queries
    waiting for its model are answered with the fit's error."""

    def __init__(self, budget_bytes: int, max_slots: int = 8, max_batch_molecules: int = 8192,
                 model_sizes: Optional[Dict[str, int]] = None,
                 model_kinds: Optional[Dict[str, str]] = None):
        self.budget = int(budget_bytes)
        self.max_slots = max_slots
        self.max_batch = max_batch_molecules
        self.queue: "collections.deque[Request]" = collections.deque()
        self.in_use = 0
        self.slots = 0
        self.fit_running = False
        self.model_sizes: Dict[str, int] = dict(model_sizes or {})
        self.model_kinds: Dict[str, str] = dict(model_kinds or {})
        self.failed_models: Dict[str, str] = {}
        self.in_use = sum(resident_bytes(n) for n in self.model_sizes.values())
        self._held: Dict[int, int] = {}   # admitted cost per unit of work (first request's id)

    def _predict_cost(self, model: str, mols: int) -> int:
        return predict_bytes(mols, self.model_sizes.get(model, 0),
                             self.model_kinds.get(model, "gaussian"))

    def submit(self, req: Request):
        self.queue.append(req)

    def cost(self, req: Request) -> int:
        if req.kind == "fit":
            return fit_bytes(req.n_mol, req.kernel)
        return self._predict_cost(req.model, req.n_mol)

    def next_batch(self) -> Optional[List[Request]]:
        """The next admissible unit of work, or None.  Fits go one at a time (one
        worker); predictions of the head request's model are merged in arrival
        order up to the molecule cap.  A request that does not fit the budget
        waits; one that can never fit is rejected."""
        if not self.queue:
            return None
        head = self.queue[0]
        if head.kind == "predict" and head.model in self.failed_models:
            self.queue.popleft()
            head.error = "model %r failed to fit: %s" % (head.model,
                                                         self.failed_models[head.model])
            return [head]
        if head.kind == "predict" and head.model not in self.model_sizes:
            # its model is still being fitted: look for other work behind it
            for k, r in enumerate(self.queue):
                if r.kind == "fit" or r.model in self.model_sizes or r.model in self.failed_models:
                    self.queue.rotate(-k)
                    return self.next_batch()
            else:
                return None
        cost = self.cost(head)
        if cost > self.budget:
            self.queue.popleft()
            head.error = "request needs %d bytes, budget is %d" % (cost, self.budget)
            if head.kind == "fit":
                self.failed_models[head.model] = head.error
            return [head]
        if head.kind == "fit":
            if self.fit_running or self.in_use + cost > self.budget:
                # let predictions behind it proceed
                for k, r in enumerate(self.queue):
                    if r.kind == "predict" and r.model in self.model_sizes:
                        self.queue.rotate(-k)
                        return self.next_batch_predict()
                return None
            self.queue.popleft()
            self.in_use += cost
            self._held[id(head)] = cost
            self.fit_running = True
            return [head]
        return self.next_batch_predict()

    def next_batch_predict(self) -> Optional[List[Request]]:
        if self.slots >= self.max_slots or not self.queue:
            return None
        head = self.queue[0]
        batch, mols = [], 0
        rest = collections.deque()
        while self.queue:
            r = self.queue.popleft()
            if (r.kind == "predict" and r.model == head.model
                    and (not batch or mols + r.n_mol <= self.max_batch)):
                batch.append(r)
                mols += r.n_mol
            else:
                rest.append(r)
        self.queue = rest + self.queue
        cost = self._predict_cost(head.model, mols)
        if self.in_use + cost > self.budget:
            for r in reversed(batch):
                self.queue.appendleft(r)
            return None
        self.in_use += cost
        self._held[id(batch[0])] = cost
        self.slots += 1
        return batch

    def release(self, batch: List[Request]):
        if not batch:
            return
        held = self._held.pop(id(batch[0]), 0)
        if batch[0].kind == "fit":
            self.in_use -= held
            self.fit_running = False
            if batch[0].error is None:
                self.model_sizes[batch[0].model] = batch[0].n_mol
                self.model_kinds[batch[0].model] = batch[0].kernel
                self.in_use += resident_bytes(batch[0].n_mol)
            else:
                self.failed_models[batch[0].model] = batch[0].error
        else:
            self.in_use -= held
            self.slots -= 1


def merge_molecules(batch: List[Request]):
    """Concatenate the ragged molecule arrays of a batch; returns flat arrays and
    the molecule range of each request."""
    charges = np.concatenate([r.charges for r in batch])
    coords = np.concatenate([r.coordinates for r in batch])
    offsets = [np.zeros(1, dtype=np.int64)]
    ranges, atom_base, mol_base = [], 0, 0
    for r in batch:
        offsets.append(r.offsets[1:] + atom_base)
        atom_base += int(r.offsets[-1])
        ranges.append((mol_base, mol_base + r.n_mol))
        mol_base += r.n_mol
    return charges, coords, np.concatenate(offsets).astype(np.int64), ranges


class GpuExecutor:
    """Runs prediction batches and fits on the GPU through qml_gb300.core.

    Every prediction slot owns a CUDA stream and preallocated pinned staging
    buffers sized for max_batch_molecules.  Query launches therefore never
    allocate pinned host memory; such allocations can synchronise the whole
    device, and a query would then wait behind a running fit."""

    def __init__(self, device="cuda", n_streams: int = 8, precision: str = "mixed",
                 fit_sm_fraction: float = 0.75, max_batch_molecules: int = 8192,
                 max_atoms: int = 23):
        import torch
        from . import core
        self.torch = torch
        self.core = core
        self.device = torch.device(device)
        # queries on high-priority streams; fits on a low-priority one, with their
        # persistent kernels capped below the SM count (fit_sm_fraction) so that
        # query kernels find free SMs while a factorisation runs
        lo, hi = torch.cuda.Stream.priority_range()
        self.streams = [torch.cuda.Stream(self.device, priority=hi) for _ in range(n_streams)]
        self.fit_stream = torch.cuda.Stream(self.device, priority=lo)
        self.fit_sm_fraction = fit_sm_fraction
        self.precision = precision
        self.models: Dict[str, tuple] = {}
        self.lock = threading.Lock()
        self.max_mols = max_batch_molecules
        atoms = max_batch_molecules * max_atoms
        self.staging = []
        for _ in range(n_streams):
            self.staging.append({
                "charges": torch.empty(atoms, dtype=torch.float64).pin_memory(),
                "coords": torch.empty(atoms * 3, dtype=torch.float64).pin_memory(),
                "offsets": torch.empty(max_batch_molecules + 1, dtype=torch.int64).pin_memory(),
                "out": torch.empty(max_batch_molecules, dtype=torch.float64).pin_memory(),
                "flag": torch.zeros(1, dtype=torch.int32).pin_memory(),
                "dflag": torch.zeros(1, dtype=torch.int32, device=self.device),
            })
        self.free = list(range(n_streams))

    def add_model(self, name, X, alpha, sigma, kernel: str = "gaussian"):
        if kernel not in ("gaussian", "laplacian"):
            raise ValueError("unknown kernel %r" % (kernel,))
        with self.lock:
            self.models[name] = (X, alpha, sigma, kernel)

    def set_query_persistence(self, on: bool):
        """Query kernels are launched from the serving thread: one CTA per tile
        while serving (they share the GPU with fits), persistent otherwise."""
        self.core.lib().qmlg_set_thread_persistent(1 if on else 0)

    def launch_predict(self, batch: List[Request]):
        """Enqueue one merged prediction on a free slot; returns (event, finish)
        where finish() copies the results into the requests once the event has
        completed and frees the slot.  If the launch fails (an allocation, for
        example), the slot's stream is drained and the slot freed before the error
        propagates, so its staging buffers are never rewritten under a copy."""
        slot = self.free.pop()
        try:
            return self._launch_on(slot, batch)
        except Exception:
            self.streams[slot].synchronize()
            self.free.append(slot)
            raise

    def _launch_on(self, slot: int, batch: List[Request]):
        torch = self.torch
        stream, st = self.streams[slot], self.staging[slot]
        with self.lock:
            X, alpha, sigma, kernel = self.models[batch[0].model]
        charges, coords, offsets, ranges = merge_molecules(batch)
        n, na = offsets.shape[0] - 1, charges.shape[0]
        if n > self.max_mols or na * 3 > st["coords"].numel():
            raise ValueError("batch larger than the staging buffers")
        st["charges"].numpy()[:na] = charges
        st["coords"].numpy()[:3 * na] = coords.reshape(-1)
        st["offsets"].numpy()[:n + 1] = offsets
        with torch.cuda.stream(stream):
            z = st["charges"][:na].to(self.device, non_blocking=True)
            r = st["coords"][:3 * na].to(self.device, non_blocking=True).view(na, 3)
            o = st["offsets"][:n + 1].to(self.device, non_blocking=True)
            Xq = self.core.coulomb_matrix_batch_async(z, r, o, CM_SIZE)
            fast = self.precision == "mixed"
            if fast:
                st["dflag"].zero_()
                if kernel == "laplacian":
                    y = self.core.predict_laplacian_async(X, Xq, sigma, alpha, st["dflag"])
                else:
                    y = self.core.predict_async(X, Xq, sigma, alpha, st["dflag"])
                st["flag"].copy_(st["dflag"], non_blocking=True)
            else:
                y = self.core.predict(kernel, X, Xq, sigma, alpha)
            st["out"][:n].copy_(y, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)

        def finish():
            try:
                vals = st["out"].numpy()[:n]
                flag = int(st["flag"][0]) if fast else 0
                path = ("fixed" if kernel == "laplacian" else "tensor") if fast else "fp64"
                if kernel == "laplacian" and flag & 8:
                    # the fixed-point bound was not met: the FP64 kernel launched
                    # beside it already wrote the result
                    path = "fp64"
                elif flag != 0:
                    # the tensor-core bound was not met (or a bounded wait gave up):
                    # recompute this batch with the FP64 kernel
                    with torch.cuda.stream(stream):
                        vals = self.core.predict(kernel, X, Xq, sigma, alpha).cpu().numpy()
                    path = "fp64"
                for req, (a, b) in zip(batch, ranges):
                    req.result = vals[a:b].copy()
                    req.path, req.flag = path, flag
            finally:
                self.free.append(slot)
        return ev, finish

    def run_fit(self, req: Request):
        """Blocking fit on the fit stream (called from the worker thread)."""
        torch = self.torch
        from .krr import KRR
        if self.fit_sm_fraction < 1.0:  # per host thread: set it on the thread that fits
            sms = torch.cuda.get_device_properties(self.device).multi_processor_count
            self.core.lib().qmlg_set_thread_sm_limit(max(2, int(sms * self.fit_sm_fraction)))
        with torch.cuda.stream(self.fit_stream):
            # pageable copies: they block this worker thread only
            z = torch.from_numpy(np.ascontiguousarray(req.charges)).to(self.device)
            r = torch.from_numpy(np.ascontiguousarray(req.coordinates)).to(self.device)
            o = torch.from_numpy(np.ascontiguousarray(req.offsets)).to(self.device)
            y = torch.from_numpy(np.ascontiguousarray(req.labels)).to(self.device)
            X = self.core.coulomb_matrix_batch(z, r, o, CM_SIZE)
            m = KRR(kernel=req.kernel, sigma=req.sigma, lam=req.lam,
                    precision=self.precision).fit(X, y)
            self.fit_stream.synchronize()
        self.add_model(req.model, X, m.alpha, req.sigma, req.kernel)
        req.result = np.array([m.report.get("outer_iterations", 0)], dtype=np.float64)


class Server:
    """The continuous-batching loop.  `clock` returns seconds."""

    def __init__(self, executor, scheduler: Scheduler, clock: Callable[[], float] = time.perf_counter):
        self.ex = executor
        self.sched = scheduler
        self.clock = clock
        self.inflight = []          # (event, finish, batch)
        self.fit_q: "queue.Queue" = queue.Queue()
        self.fit_done: "queue.Queue" = queue.Queue()
        self.worker = threading.Thread(target=self._fit_worker, daemon=True)
        self.worker.start()
        self.completed: List[Request] = []

    def _fit_worker(self):
        while True:
            batch = self.fit_q.get()
            if batch is None:
                return
            try:
                self.ex.run_fit(batch[0])
            except Exception as e:  # reported on the request, the server keeps going
                batch[0].error = repr(e)
            batch[0].done = self.clock()
            self.fit_done.put(batch)

    def _retire(self):
        still = []
        for ev, finish, batch in self.inflight:
            if ev.query():
                try:
                    finish()
                except Exception as e:  # reported on the requests, the server keeps going
                    for r in batch:
                        r.error, r.result = repr(e), None
                t = self.clock()
                for r in batch:
                    r.done = t
                self.sched.release(batch)
                self.completed.extend(batch)
            else:
                still.append((ev, finish, batch))
        self.inflight = still
        while not self.fit_done.empty():
            batch = self.fit_done.get()
            self.sched.release(batch)
            self.completed.extend(batch)

    def _admit(self):
        while True:
            batch = self.sched.next_batch()
            if batch is None:
                return
            t = self.clock()
            for r in batch:
                r.admitted = t
            if batch[0].error is not None:
                batch[0].done = t
                self.completed.append(batch[0])
                continue
            if batch[0].kind == "fit":
                self.fit_q.put(batch)
                continue
            try:
                ev, finish = self.ex.launch_predict(batch)
            except Exception as e:  # reported on the requests, the server keeps going
                for r in batch:
                    r.error, r.done = repr(e), t
                self.sched.release(batch)
                self.completed.extend(batch)
                continue
            self.inflight.append((ev, finish, batch))

    def run(self, arrivals: List[Request], idle_sleep: float = 50e-6) -> List[Request]:
        """Serve `arrivals` (sorted by arrival time, relative to start) to completion."""
        set_persistent = getattr(self.ex, "set_query_persistence", None)
        if set_persistent is not None:
            set_persistent(False)
        try:
            return self._run(arrivals, idle_sleep)
        finally:
            if set_persistent is not None:
                set_persistent(True)

    def _run(self, arrivals: List[Request], idle_sleep: float) -> List[Request]:
        t0 = self.clock()
        pending = collections.deque(sorted(arrivals, key=lambda r: r.arrival))
        total = len(pending)
        for r in pending:
            r.arrival += t0
        while len(self.completed) < total:
            now = self.clock()
            while pending and pending[0].arrival <= now:
                self.sched.submit(pending.popleft())
            self._retire()
            self._admit()
            if not self.inflight and self.sched.queue == collections.deque() and pending:
                time.sleep(max(0.0, min(idle_sleep, pending[0].arrival - self.clock())))
            elif self.inflight:
                time.sleep(idle_sleep)
        self.fit_q.put(None)
        return self.completed


def poisson_workload(rate_hz: float, duration_s: float, pool, model: str,
                     fit_every: int = 0, fit_sizes=(1000, 20000), seed: int = 0,
                     max_query: int = 4096, fit_kernel: str = "gaussian",
                     fit_sigma: float = 1000.0) -> List[Request]:
    """Poisson arrivals of prediction queries (molecule count log-uniform in
    1..max_query) and, every `fit_every`-th arrival, a fit request with N
    log-uniform in fit_sizes (kernel fit_kernel, width fit_sigma).  Molecules are
    consecutive slices of `pool` (a MoleculeBatch with labels) starting at random
    offsets."""
    rng = np.random.default_rng(seed)
    t, rid, out = 0.0, 0, []

    def take(n):
        n = min(max(1, n), pool.n_mol)
        start = int(rng.integers(0, pool.n_mol - n + 1))
        return pool.slice(start, start + n)

    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > duration_s:
            break
        if fit_every and rid % fit_every == fit_every - 1:
            n = int(round(math.exp(rng.uniform(math.log(fit_sizes[0]), math.log(fit_sizes[1])))))
            b = take(n)
            out.append(Request(rid, "fit", "fit-%d" % rid, b.charges, b.coordinates, b.offsets, t,
                               labels=b.labels, kernel=fit_kernel, sigma=fit_sigma))
        else:
            n = int(round(math.exp(rng.uniform(0.0, math.log(max_query)))))
            b = take(n)
            out.append(Request(rid, "predict", model, b.charges, b.coordinates, b.offsets, t))
        rid += 1
    return out


def latency_stats(done: List[Request]) -> dict:
    preds = [r for r in done if r.kind == "predict" and r.error is None]
    fits = [r for r in done if r.kind == "fit" and r.error is None]
    lat = np.array([r.latency for r in preds]) if preds else np.zeros(0)
    span = (max(r.done for r in done) - min(r.arrival for r in done)) if done else 0.0
    mols = sum(r.n_mol for r in preds)
    return {
        "queries": len(preds), "fits": len(fits),
        "rejected": sum(1 for r in done if r.error is not None),
        "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
        "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
        "mean_ms": float(lat.mean() * 1e3) if lat.size else None,
        "molecules_per_s": mols / span if span > 0 else None,
        "fit_latency_ms": [float(r.latency * 1e3) for r in fits],
    }
