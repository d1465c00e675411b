"""Batched KRR fits recorded into one CUDA graph.

Learning curves and sigma x lambda grids are many independent fits of uneven size
(docs/source/tutorial.rst:168-174 of the reference).  BatchedKRR lays out one kernel
matrix, solution and status per fit and records all of them into a single CUDA graph.

mode "grouped" (default): every phase is one grouped launch over all fits
(qmlg_fit_batched_async): the tensor-core Gaussian kernel matrices of all fits in one
persistent launch whose tile list spans the fits; the mixed factorisations in
lockstep 64-column steps (the FP64 diagonal blocks of all fits in one launch, their
panel solves in one, their K = 64 updates in one tensor-core launch, and every 512
columns all trailing updates in one tensor-core launch); then the triangular solves
one 64-row block per launch for all fits, and a fixed number of exact-residual
refinement steps.

mode "streams": the earlier schedule, each fit's own launches (capture-safe kernel
matrix, qmlg_solve_async) spread over several streams forked from the capture stream.

Replaying the graph reruns every fit with one host call; the host checks the per-fit
status words afterwards.

The autotuner times graph replays over candidate tile parameters of the grouped
path (the i-columns per tensor-core tile of the factorisation's updates, 64 or 32,
and the rows per CTA of the panel solves) and keeps the fastest, cached per
(device name, size bucket): the bucket is the fit count and the power of two above
the largest fit.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib, core

_TUNED: Dict[Tuple, dict] = {}
MAX_GROUP = 128  # fits per grouped call (the C ABI's limit)


@dataclass
class Problem:
    X: torch.Tensor          # (n, d) float64 CUDA, row-major representations
    y: torch.Tensor          # (n,) float64 CUDA
    sigma: float
    lam: float
    kernel: str = "gaussian"  # or "laplacian"


def size_bucket(problems: Sequence[Problem]) -> Tuple[int, int]:
    """(fit count, power of two at or above the largest fit)."""
    nmax = max(p.X.shape[0] for p in problems)
    return len(problems), 1 << max(0, math.ceil(math.log2(max(nmax, 1))))


class BatchedKRR:
    def __init__(self, problems: Sequence[Problem], refine_steps: int = 3, mode: str = "grouped",
                 tile_cols: int = 64, trsm_rows: int = 128, streams: int = 4, order: str = "size",
                 persistent: bool = True):
        if not problems:
            raise ValueError("no problems")
        if mode not in ("grouped", "streams"):
            raise ValueError("mode must be 'grouped' or 'streams'")
        self.problems = list(problems)
        self.refine_steps = int(refine_steps)
        self.device = self.problems[0].X.device
        self.config = {"mode": mode, "tile_cols": tile_cols, "trsm_rows": trsm_rows,
                       "streams": streams, "order": order, "persistent": persistent}
        lib = core.lib()
        d = self.problems[0].X.shape[1]
        self.K, self.x, self.status, self.flag, self.corr = [], [], [], [], []
        self.ws: List[torch.Tensor] = []
        for p in self.problems:
            n, dp = p.X.shape
            if p.X.dtype != torch.float64 or p.X.stride(1) != 1 or p.y.shape != (n,) or dp != d:
                raise ValueError("X must be (n, d) row-major float64 with one d, and y (n,)")
            if p.kernel not in ("gaussian", "laplacian"):
                raise ValueError("unknown kernel %r" % (p.kernel,))
            self.K.append(torch.empty((n, n), dtype=torch.float64, device=self.device))
            self.x.append(torch.empty(n, dtype=torch.float64, device=self.device))
            self.status.append(torch.zeros(2, dtype=torch.int32, device=self.device))
            self.flag.append(torch.zeros(1, dtype=torch.int32, device=self.device))
            self.corr.append(torch.zeros(2, dtype=torch.float64, device=self.device))
        self.d = d
        self._groups: List[Tuple[List[int], ctypes.Array, torch.Tensor]] = []
        self._stream_ws: Optional[List[torch.Tensor]] = None
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self._streams: List[torch.cuda.Stream] = []

    # ------------------------------------------------------ grouped layout --
    def _grouped_calls(self):
        """The problem tables and workspaces of the grouped calls (built once)."""
        if self._groups:
            return self._groups
        lib = core.lib()
        order = list(range(len(self.problems)))
        order.sort(key=lambda i: -self.problems[i].X.shape[0])  # largest first
        for start in range(0, len(order), MAX_GROUP):
            idx = order[start:start + MAX_GROUP]
            arr = (_lib.QmlgBatchProblem * len(idx))()
            for k, i in enumerate(idx):
                p = self.problems[i]
                n = p.X.shape[0]
                arr[k] = _lib.QmlgBatchProblem(
                    p.X.data_ptr(), p.X.stride(0), n,
                    _lib.QMLG_KIND_GAUSSIAN if p.kernel == "gaussian" else _lib.QMLG_KIND_LAPLACIAN,
                    float(p.sigma), float(p.lam), p.y.data_ptr(), self.x[i].data_ptr(),
                    self.K[i].data_ptr(), self.status[i].data_ptr(), self.corr[i].data_ptr())
            nbytes = lib.qmlg_fit_batched_workspace_size(arr, len(idx), self.d)
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._groups.append((idx, arr, ws))
        return self._groups

    def _enqueue_grouped(self):
        lib = core.lib()
        s = torch.cuda.current_stream(self.device).cuda_stream
        for idx, arr, ws in self._grouped_calls():
            _lib.check(lib.qmlg_fit_batched_async(arr, len(idx), self.d, self.refine_steps,
                                                  int(self.config["tile_cols"]),
                                                  int(self.config["trsm_rows"]), ws.data_ptr(),
                                                  ws.numel(), s), "qmlg_fit_batched_async")

    # ------------------------------------------------------- stream layout --
    def _order(self) -> List[int]:
        idx = list(range(len(self.problems)))
        if self.config["order"] == "size":
            idx.sort(key=lambda i: -self.problems[i].X.shape[0])
        return idx

    def _enqueue_one(self, i: int):
        lib = core.lib()
        if self._stream_ws is None:
            self._stream_ws = []
            for p in self.problems:
                n, d = p.X.shape
                size_fn = (lib.qmlg_gaussian_kernel_emulated_workspace_size
                           if p.kernel == "gaussian" else
                           lib.qmlg_laplacian_kernel_fixed_workspace_size)
                nbytes = max(size_fn(n, n, d, _lib.QMLG_KERNEL_SYMMETRIC),
                             lib.qmlg_solve_async_workspace_size(n))
                self._stream_ws.append(torch.empty(nbytes, dtype=torch.uint8, device=self.device))
        p = self.problems[i]
        n, d = p.X.shape
        s = torch.cuda.current_stream(self.device).cuda_stream
        K, ws = self.K[i], self._stream_ws[i]
        self.flag[i].zero_()
        fn, name = ((lib.qmlg_gaussian_kernel_emulated_async, "qmlg_gaussian_kernel_emulated_async")
                    if p.kernel == "gaussian" else
                    (lib.qmlg_laplacian_kernel_fixed_async, "qmlg_laplacian_kernel_fixed_async"))
        _lib.check(fn(p.X.data_ptr(), p.X.stride(0), n, p.X.data_ptr(), p.X.stride(0), n, d,
                      float(p.sigma), K.data_ptr(), n, _lib.QMLG_KERNEL_SYMMETRIC, 0.0,
                      self.flag[i].data_ptr(), ws.data_ptr(), ws.numel(), s), name)
        _lib.check(lib.qmlg_solve_async(
            K.data_ptr(), n, n, p.y.data_ptr(), self.x[i].data_ptr(), float(p.lam),
            self.refine_steps, self.status[i].data_ptr(), self.corr[i].data_ptr(),
            ws.data_ptr(), ws.numel(), s), "qmlg_solve_async")

    def _enqueue_streams(self):
        main = torch.cuda.current_stream(self.device)
        ns = max(1, min(self.config["streams"], len(self.problems)))
        while len(self._streams) < ns:
            self._streams.append(torch.cuda.Stream(self.device))
        lib = core.lib()
        lib.qmlg_set_thread_persistent(1 if self.config["persistent"] else 0)
        try:
            for s in self._streams[:ns]:
                s.wait_stream(main)
            for k, i in enumerate(self._order()):
                with torch.cuda.stream(self._streams[k % ns]):
                    self._enqueue_one(i)
            for s in self._streams[:ns]:
                main.wait_stream(s)
        finally:
            lib.qmlg_set_thread_persistent(1)

    # ------------------------------------------------------------ recording --
    def _enqueue_all(self):
        lib = core.lib()
        lib.qmlg_set_thread_cooperative(0)  # concurrent solves: no grid-wide waits
        try:
            if self.config["mode"] == "grouped":
                for f in self.flag:
                    f.zero_()
                self._enqueue_grouped()
            else:
                self._enqueue_streams()
        finally:
            lib.qmlg_set_thread_cooperative(1)

    def run_eager(self):
        self._enqueue_all()
        torch.cuda.synchronize(self.device)

    def capture(self):
        """Record every fit into one CUDA graph (after one eager warm-up run, which
        also performs the library's one-time set-up outside the capture)."""
        self.run_eager()
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream(self.device)
        cap.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap):
                self._enqueue_all()
        torch.cuda.current_stream(self.device).wait_stream(cap)
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    # ------------------------------------------------------------- results --
    def results(self):
        """(alpha list, report list) after the work has completed.  "flags" nonzero
        means the fit needs a rerun (a bounded wait gave up, or the Gaussian
        tensor-core bound failed); "kernel_path" says which kernel formed K (a
        Laplacian whose fixed-point bound failed was formed by the FP64 kernel in
        the same graph, which is not an error)."""
        torch.cuda.synchronize(self.device)
        reports = []
        for i, p in enumerate(self.problems):
            st = self.status[i].cpu().tolist()
            fl = int(self.flag[i].item()) | st[1]
            c = self.corr[i].cpu().tolist()
            if p.kernel == "laplacian":
                path = "fp64" if fl & 8 else "fixed"
                fl &= ~8
            else:
                path = "tensor"
            reports.append({"info": st[0], "flags": fl, "kernel_path": path,
                            "last_correction": (c[0] ** 0.5) / max(c[1] ** 0.5, 1e-300)})
        return self.x, reports

    # ------------------------------------------------------------ autotuning --
    def autotune(self, candidates=None, reps: int = 2) -> dict:
        """Time graph replays for each candidate configuration and keep the fastest.
        Default candidates: the grouped path with tile_cols in {64, 32} and
        trsm_rows in {64, 128}.  Cached per (device name, size bucket)."""
        key = (torch.cuda.get_device_name(self.device), size_bucket(self.problems))
        if key in _TUNED:
            self.config = dict(_TUNED[key])
            self.graph = None
            return dict(self.config)
        if candidates is None:
            candidates = [{"mode": "grouped", "tile_cols": tc, "trsm_rows": tr}
                          for tc in (64, 32) for tr in (128, 64)]
        best, best_t = None, float("inf")
        for cfg in candidates:
            self.config = dict(self.config, **cfg)
            self.graph = None
            self.capture()
            start = torch.cuda.Event(enable_timing=True)
            stop = torch.cuda.Event(enable_timing=True)
            start.record()
            for _ in range(reps):
                self.graph.replay()
            stop.record()
            torch.cuda.synchronize(self.device)
            t = start.elapsed_time(stop) / reps
            if t < best_t:
                best, best_t = dict(self.config), t
        self.config = best
        self.graph = None
        _TUNED[key] = dict(best)
        return dict(best, ms=best_t)
