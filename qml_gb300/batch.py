"""Batched KRR fits recorded into one CUDA graph.

Learning curves and sigma x lambda grids are many independent fits of uneven size.
BatchedKRR lays out one kernel matrix, workspace and solution per fit, then records
all of them into a single CUDA graph.  The fits are spread over several streams
forked from the capture stream.  Each fit is a capture-safe kernel matrix (the
tensor-core Gaussian, qmlg_gaussian_kernel_emulated_async, or the fixed-point
Laplacian, qmlg_laplacian_kernel_fixed_async) followed by the capture-safe mixed
solve (qmlg_solve_async) with a fixed number of exact-residual refinement steps.
Replaying the graph reruns every fit with one host call; the host checks the
per-fit status words afterwards.

The autotuner times graph replays over a small set of scheduling choices and
keeps the fastest:
  * streams: how many fits run concurrently;
  * order: largest fits first, or round-robin;
  * persistent: persistent CTAs, or one CTA per tile for the tensor-core kernels.
The choice is cached per (device, sorted problem sizes).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib, core

_TUNED: Dict[Tuple, dict] = {}


@dataclass
class Problem:
    X: torch.Tensor          # (n, d) float64 CUDA, row-major representations
    y: torch.Tensor          # (n,) float64 CUDA
    sigma: float
    lam: float
    kernel: str = "gaussian"  # or "laplacian"


class BatchedKRR:
    def __init__(self, problems: Sequence[Problem], refine_steps: int = 3, streams: int = 4,
                 order: str = "size", persistent: bool = True):
        if not problems:
            raise ValueError("no problems")
        self.problems = list(problems)
        self.refine_steps = int(refine_steps)
        self.device = self.problems[0].X.device
        self.config = {"streams": streams, "order": order, "persistent": persistent}
        lib = core.lib()
        self.K, self.x, self.ws, self.status, self.flag, self.corr = [], [], [], [], [], []
        for p in self.problems:
            n, d = p.X.shape
            if p.X.dtype != torch.float64 or p.X.stride(1) != 1 or p.y.shape != (n,):
                raise ValueError("X must be (n, d) row-major float64 and y (n,)")
            if p.kernel not in ("gaussian", "laplacian"):
                raise ValueError("unknown kernel %r" % (p.kernel,))
            size_fn = (lib.qmlg_gaussian_kernel_emulated_workspace_size if p.kernel == "gaussian"
                       else lib.qmlg_laplacian_kernel_fixed_workspace_size)
            ws_bytes = max(size_fn(n, n, d, _lib.QMLG_KERNEL_SYMMETRIC),
                           lib.qmlg_solve_async_workspace_size(n))
            self.K.append(torch.empty((n, n), dtype=torch.float64, device=self.device))
            self.x.append(torch.empty(n, dtype=torch.float64, device=self.device))
            self.ws.append(torch.empty(ws_bytes, dtype=torch.uint8, device=self.device))
            self.status.append(torch.zeros(2, dtype=torch.int32, device=self.device))
            self.flag.append(torch.zeros(1, dtype=torch.int32, device=self.device))
            self.corr.append(torch.zeros(2, dtype=torch.float64, device=self.device))
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self._streams: List[torch.cuda.Stream] = []

    # ------------------------------------------------------------ recording --
    def _order(self) -> List[int]:
        idx = list(range(len(self.problems)))
        if self.config["order"] == "size":
            idx.sort(key=lambda i: -self.problems[i].X.shape[0])
        return idx

    def _enqueue_one(self, i: int):
        lib = core.lib()
        p = self.problems[i]
        n, d = p.X.shape
        s = torch.cuda.current_stream(self.device).cuda_stream
        K = self.K[i]
        self.flag[i].zero_()
        fn, name = ((lib.qmlg_gaussian_kernel_emulated_async, "qmlg_gaussian_kernel_emulated_async")
                    if p.kernel == "gaussian" else
                    (lib.qmlg_laplacian_kernel_fixed_async, "qmlg_laplacian_kernel_fixed_async"))
        _lib.check(fn(p.X.data_ptr(), p.X.stride(0), n, p.X.data_ptr(), p.X.stride(0), n, d,
                      float(p.sigma), K.data_ptr(), n, _lib.QMLG_KERNEL_SYMMETRIC, 0.0,
                      self.flag[i].data_ptr(), self.ws[i].data_ptr(), self.ws[i].numel(), s), name)
        _lib.check(lib.qmlg_solve_async(
            K.data_ptr(), n, n, p.y.data_ptr(), self.x[i].data_ptr(), float(p.lam),
            self.refine_steps, self.status[i].data_ptr(), self.corr[i].data_ptr(),
            self.ws[i].data_ptr(), self.ws[i].numel(), s), "qmlg_solve_async")

    def _enqueue_all(self):
        """Fork the streams from the current stream, enqueue the fits, join back."""
        main = torch.cuda.current_stream(self.device)
        ns = max(1, min(self.config["streams"], len(self.problems)))
        while len(self._streams) < ns:
            self._streams.append(torch.cuda.Stream(self.device))
        lib = core.lib()
        lib.qmlg_set_thread_persistent(1 if self.config["persistent"] else 0)
        lib.qmlg_set_thread_cooperative(0)  # concurrent solves: single-CTA triangular solves
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
            fl = int(self.flag[i].item())
            c = self.corr[i].cpu().tolist()
            if p.kernel == "laplacian":
                path = "fp64" if fl & 8 else "fixed"
                fl &= ~8
            else:
                path = "tensor"
            reports.append({"info": st[0], "flags": st[1] | fl, "kernel_path": path,
                            "last_correction": (c[0] ** 0.5) / max(c[1] ** 0.5, 1e-300)})
        return self.x, reports

    # ------------------------------------------------------------ autotuning --
    def autotune(self, candidates=None, reps: int = 2) -> dict:
        """Time graph replays for each scheduling choice and keep the fastest.
        Cached per (device name, sorted problem sizes and kernels)."""
        key = (torch.cuda.get_device_name(self.device),
               tuple(sorted((p.X.shape[0], p.kernel) for p in self.problems)))
        if key in _TUNED:
            self.config = dict(_TUNED[key])
            self.graph = None
            return self.config
        if candidates is None:
            candidates = [{"streams": s, "order": o, "persistent": pm}
                          for s in (2, 4, 8) for o in ("size", "rr") for pm in (True, False)]
        best, best_t = None, float("inf")
        for cfg in candidates:
            self.config = dict(cfg)
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
                best, best_t = dict(cfg), t
        self.config = best
        self.graph = None
        _TUNED[key] = dict(best)
        return dict(best, ms=best_t)
