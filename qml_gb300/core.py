"""Device-tensor API over the C ABI (torch tensors in HBM, work on the current stream).

Every function here calls libqmlg.so; torch only provides device memory, streams
and the workspace buffers that the C ABI asks for (the library itself allocates
nothing).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import torch

from . import _lib
from ._lib import QmlgRefineOpts, QmlgSolveReport, check

_SORTING = {"row-norm": 1, "unsorted": 0}
_KINDS = {"gaussian": _lib.QMLG_KIND_GAUSSIAN, "laplacian": _lib.QMLG_KIND_LAPLACIAN}
_PRECISIONS = {"fp64": _lib.QMLG_PREC_FP64, "mixed": _lib.QMLG_PREC_MIXED}


def lib():
    return _lib.load()


def _stream(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _require_cuda(*tensors):
    for t in tensors:
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise TypeError("expected CUDA tensors")
        if t.dtype not in (torch.float64, torch.int64, torch.int32, torch.uint8):
            raise TypeError("unexpected dtype %s" % t.dtype)


class _WorkspaceCache:
    """One growing scratch buffer per (device, stream), reused across calls."""

    def __init__(self):
        self._buf = {}

    def get(self, nbytes: int, device) -> torch.Tensor:
        # one buffer per (device, stream): work queued on different streams never
        # shares scratch memory
        dev = torch.device(device)
        index = dev.index if dev.index is not None else torch.cuda.current_device()
        key = (index, torch.cuda.current_stream(index).cuda_stream)
        buf = self._buf.get(key)
        if buf is None or buf.numel() < nbytes:
            # drop the smaller buffer first: it was allocated on this stream, so the
            # allocator may hand its memory to the next allocation on this stream, and
            # the peak is the larger size rather than the sum of both
            self._buf.pop(key, None)
            del buf
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
            self._buf[key] = buf
        return buf


workspaces = _WorkspaceCache()


# ------------------------------------------------------------ Coulomb matrix --

def coulomb_matrix_batch(charges: torch.Tensor, coordinates: torch.Tensor,
                         offsets: torch.Tensor, size: int = 23,
                         sorting: str = "row-norm", out: Optional[torch.Tensor] = None
                         ) -> torch.Tensor:
    """Sorted (or unsorted) Coulomb matrices of a ragged batch of molecules.

    charges (total_atoms,) float64, coordinates (total_atoms, 3) float64,
    offsets (n_mol + 1,) int64 on the GPU -> (n_mol, size*(size+1)//2) float64.
    """
    if sorting not in _SORTING:
        raise ValueError("Unknown sorting scheme requested: %r" % (sorting,))
    _require_cuda(charges, coordinates, offsets)
    charges = charges.contiguous()
    coordinates = coordinates.contiguous()
    offsets = offsets.to(torch.int64).contiguous()
    n_mol = offsets.shape[0] - 1
    length = size * (size + 1) // 2
    if out is None:
        out = torch.empty((n_mol, length), dtype=torch.float64, device=charges.device)
    status = torch.zeros(1, dtype=torch.int32, device=charges.device)
    check(lib().qmlg_coulomb_matrix(charges.data_ptr(), coordinates.data_ptr(),
                                    offsets.data_ptr(), n_mol, size, _SORTING[sorting],
                                    out.data_ptr(), status.data_ptr(), _stream(charges.device)),
          "qmlg_coulomb_matrix")
    # wait for the stream before reading back (a read queued behind pending work
    # would hold up other host threads' CUDA calls until that work finishes)
    torch.cuda.current_stream(charges.device).synchronize()
    st = int(status.item())
    if st != 0:
        _lib.check(st, "qmlg_coulomb_matrix")
    return out


def atomic_coulomb_matrix_batch(charges: torch.Tensor, coordinates: torch.Tensor,
                                offsets: torch.Tensor, size: int = 23,
                                sorting: str = "distance", central_cutoff: float = 1e6,
                                central_decay: float = -1.0, interaction_cutoff: float = 1e6,
                                interaction_decay: float = -1.0,
                                central_offsets: Optional[torch.Tensor] = None,
                                central_atoms: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Atomic Coulomb matrices of a ragged batch: one row per central atom (every
    atom, or central_atoms grouped by central_offsets), (n_central,
    size*(size+1)//2) float64 on the GPU.  sorting "row-norm" or "distance"."""
    if sorting not in ("row-norm", "distance"):
        raise ValueError("Unknown sorting scheme requested: %r" % (sorting,))
    _require_cuda(charges, coordinates, offsets)
    charges = charges.contiguous()
    coordinates = coordinates.contiguous()
    offsets = offsets.to(torch.int64).contiguous()
    n_mol = offsets.shape[0] - 1
    if central_atoms is None:
        n_central = int(charges.shape[0])
        co = ca = None
    else:
        central_offsets = central_offsets.to(device=charges.device, dtype=torch.int64).contiguous()
        central_atoms = central_atoms.to(device=charges.device, dtype=torch.int32).contiguous()
        n_central = int(central_atoms.shape[0])
        co, ca = central_offsets.data_ptr(), central_atoms.data_ptr()
    out = torch.empty((n_central, size * (size + 1) // 2), dtype=torch.float64,
                      device=charges.device)
    status = torch.zeros(1, dtype=torch.int32, device=charges.device)
    check(lib().qmlg_atomic_coulomb_matrix(charges.data_ptr(), coordinates.data_ptr(),
                                           offsets.data_ptr(), n_mol, co, ca, n_central, size,
                                           1 if sorting == "row-norm" else 0,
                                           float(central_cutoff), float(central_decay),
                                           float(interaction_cutoff), float(interaction_decay),
                                           out.data_ptr(), status.data_ptr(),
                                           _stream(charges.device)),
          "qmlg_atomic_coulomb_matrix")
    torch.cuda.current_stream(charges.device).synchronize()
    st = int(status.item())
    if st != 0:
        _lib.check(st, "qmlg_atomic_coulomb_matrix")
    return out


def local_kernels(kind: str, A: torch.Tensor, B: torch.Tensor, offsets_a: torch.Tensor,
                  offsets_b: torch.Tensor, sigmas, symmetric: bool = False,
                  emulated: bool = False) -> torch.Tensor:
    """Local kernels (nsigmas, nm1, nm2) float64 on the GPU (a Fortran-ordered view)
    for atom rows A, B grouped by molecule offsets.  kind "gaussian" or "laplacian".
    emulated=True sums atom-pair kernel matrices from the tensor-core Gaussian or the
    fixed-point Laplacian (qmlg_local_kernels_emulated, within 1e-12 per entry)."""
    if kind not in ("gaussian", "laplacian"):
        raise ValueError("unknown local kernel %r" % (kind,))
    _require_cuda(A, B)
    A, lda = _rows(A)
    if symmetric:
        B, ldb, offsets_b = A, lda, offsets_a
    else:
        B, ldb = _rows(B)
    if A.shape[1] != B.shape[1]:
        raise ValueError("A and B have different representation sizes")
    offsets_a = offsets_a.to(device=A.device, dtype=torch.int64).contiguous()
    offsets_b = offsets_a if symmetric else offsets_b.to(device=A.device, dtype=torch.int64).contiguous()
    sg = torch.as_tensor(sigmas, dtype=torch.float64).reshape(-1).to(A.device).contiguous()
    nm1, nm2, ns = offsets_a.shape[0] - 1, offsets_b.shape[0] - 1, sg.shape[0]
    buf = torch.zeros((nm2, nm1, ns), dtype=torch.float64, device=A.device)
    if emulated:
        kc = 0 if kind == "gaussian" else 1
        # the atom counts the library sizes its chunks by (it reads the offsets too)
        nat_a, nat_b = int(offsets_a[-1]), int(offsets_b[-1])
        ws = workspaces.get(lib().qmlg_local_kernels_emulated_workspace_size(kc, nat_a, nat_b, nm2,
                                                                             A.shape[1]), A.device)
        check(lib().qmlg_local_kernels_emulated(kc, A.data_ptr(), lda, offsets_a.data_ptr(), nm1,
                                                B.data_ptr(), ldb, offsets_b.data_ptr(), nm2,
                                                A.shape[1], sg.data_ptr(), ns, buf.data_ptr(),
                                                _lib.QMLG_KERNEL_SYMMETRIC if symmetric else 0,
                                                ws.data_ptr(), ws.numel(), _stream(A.device)),
              "qmlg_local_kernels_emulated")
        return buf.permute(2, 1, 0)
    check(lib().qmlg_local_kernels(0 if kind == "gaussian" else 1, A.data_ptr(), lda,
                                   offsets_a.data_ptr(), nm1, B.data_ptr(), ldb,
                                   offsets_b.data_ptr(), nm2, A.shape[1], sg.data_ptr(), ns,
                                   buf.data_ptr(), _lib.QMLG_KERNEL_SYMMETRIC if symmetric else 0,
                                   _stream(A.device)), "qmlg_local_kernels")
    return buf.permute(2, 1, 0)


def coulomb_matrix_batch_async(charges: torch.Tensor, coordinates: torch.Tensor,
                               offsets: torch.Tensor, size: int = 23, sorting: str = "row-norm",
                               status: Optional[torch.Tensor] = None) -> torch.Tensor:
    """coulomb_matrix_batch without reading the device status back (no host
    synchronisation).  When `status` (a zeroed int32 CUDA tensor) is given, a
    molecule with too many atoms sets it to QMLG_E_TOO_MANY_ATOMS."""
    if sorting not in _SORTING:
        raise ValueError("Unknown sorting scheme requested: %r" % (sorting,))
    _require_cuda(charges, coordinates, offsets)
    n_mol = offsets.shape[0] - 1
    out = torch.empty((n_mol, size * (size + 1) // 2), dtype=torch.float64, device=charges.device)
    check(lib().qmlg_coulomb_matrix(charges.contiguous().data_ptr(),
                                    coordinates.contiguous().data_ptr(),
                                    offsets.to(torch.int64).contiguous().data_ptr(), n_mol, size,
                                    _SORTING[sorting], out.data_ptr(),
                                    status.data_ptr() if status is not None else None,
                                    _stream(charges.device)), "qmlg_coulomb_matrix")
    return out


# ------------------------------------------------------------ kernel matrices --

def _rows(X: torch.Tensor) -> Tuple[torch.Tensor, int]:
    if X.dim() != 2 or X.dtype != torch.float64:
        raise ValueError("expected a 2-D float64 representation matrix")
    if X.stride(1) != 1:
        X = X.contiguous()
    return X, max(X.stride(0), X.shape[1])


def kernel_matrix(kind: str, A: torch.Tensor, B: torch.Tensor, sigma: float,
                  symmetric: bool = False, diag_shift: float = 0.0,
                  out: Optional[torch.Tensor] = None, emulated: bool = False,
                  order: int = 0, gammas=None) -> torch.Tensor:
    """K (na, nb), Fortran-ordered like the reference, as a (na, nb) view of a
    column-major buffer.  symmetric=True requires B is A.

    kind: "gaussian", "laplacian", "linear" (sigma unused), "matern_l2" (with
    order 0/1/2) or "sargan" (with gammas, a sequence or 1-D tensor).
    emulated=True takes the fast exact-within-1e-12 paths: the Gaussian contraction
    on the tensor cores (qmlg_gaussian_kernel_emulated), the Laplacian L1 sums in
    fixed-point integers (qmlg_laplacian_kernel_fixed), the linear kernel's dot
    products and the Matern L2 orders 1 and 2 on the tensor cores
    (qmlg_linear_kernel_emulated, qmlg_matern_kernel_l2_emulated), the Sargan kernel
    from fixed-point L1 sums (qmlg_sargan_kernel_fixed); Matern order 0 takes its FP64
    kernel."""
    _require_cuda(A, B)
    A, lda = _rows(A)
    if symmetric:
        B, ldb = A, lda
    else:
        B, ldb = _rows(B)
    na, nb, d = A.shape[0], B.shape[0], A.shape[1]
    if B.shape[1] != d:
        raise ValueError("A and B have different representation sizes")
    if out is None:
        buf = torch.empty((nb, na), dtype=torch.float64, device=A.device)
    else:
        if out.shape != (na, nb) or out.stride() != (1, na):
            raise ValueError("out must be a Fortran-ordered (na, nb) float64 tensor")
        buf = out.T
    flags = _lib.QMLG_KERNEL_SYMMETRIC if symmetric else 0
    if emulated and kind == "gaussian":
        ws_bytes = lib().qmlg_gaussian_kernel_emulated_workspace_size(na, nb, d, flags)
        ws = workspaces.get(ws_bytes, A.device)
        check(lib().qmlg_gaussian_kernel_emulated(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                                  float(sigma), buf.data_ptr(), na, flags,
                                                  float(diag_shift), ws.data_ptr(), ws.numel(),
                                                  _stream(A.device)),
              "qmlg_gaussian_kernel_emulated")
        return buf.T
    if emulated and kind == "linear":
        ws_bytes = lib().qmlg_linear_kernel_emulated_workspace_size(na, nb, d, flags)
        ws = workspaces.get(ws_bytes, A.device)
        check(lib().qmlg_linear_kernel_emulated(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                                buf.data_ptr(), na, flags, float(diag_shift),
                                                ws.data_ptr(), ws.numel(), _stream(A.device)),
              "qmlg_linear_kernel_emulated")
        return buf.T
    if emulated and kind == "matern_l2":
        ws_bytes = lib().qmlg_matern_kernel_l2_emulated_workspace_size(na, nb, d, flags)
        ws = workspaces.get(ws_bytes, A.device)
        check(lib().qmlg_matern_kernel_l2_emulated(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb,
                                                   d, float(sigma), int(order), buf.data_ptr(), na,
                                                   flags, float(diag_shift), ws.data_ptr(),
                                                   ws.numel(), _stream(A.device)),
              "qmlg_matern_kernel_l2_emulated")
        return buf.T
    if emulated and kind == "laplacian":
        ws_bytes = lib().qmlg_laplacian_kernel_fixed_workspace_size(na, nb, d, flags)
        ws = workspaces.get(ws_bytes, A.device)
        check(lib().qmlg_laplacian_kernel_fixed(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                                float(sigma), buf.data_ptr(), na, flags,
                                                float(diag_shift), ws.data_ptr(), ws.numel(),
                                                _stream(A.device)),
              "qmlg_laplacian_kernel_fixed")
        return buf.T
    st = _stream(A.device)
    if kind == "linear":
        check(lib().qmlg_linear_kernel(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                       buf.data_ptr(), na, flags, float(diag_shift), st),
              "qmlg_linear_kernel")
        return buf.T
    if kind == "matern_l2":
        check(lib().qmlg_matern_kernel_l2(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                          float(sigma), int(order), buf.data_ptr(), na, flags,
                                          float(diag_shift), st), "qmlg_matern_kernel_l2")
        return buf.T
    if kind == "sargan":
        g = torch.as_tensor(gammas if gammas is not None else [], dtype=torch.float64)
        g = g.reshape(-1).to(A.device).contiguous()
        if emulated:
            ws = workspaces.get(lib().qmlg_sargan_kernel_fixed_workspace_size(na, nb, d, flags),
                                A.device)
            check(lib().qmlg_sargan_kernel_fixed(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                                 float(sigma), g.data_ptr() if g.numel() else None,
                                                 int(g.numel()), buf.data_ptr(), na, flags,
                                                 float(diag_shift), ws.data_ptr(), ws.numel(), st),
                  "qmlg_sargan_kernel_fixed")
            return buf.T
        check(lib().qmlg_sargan_kernel(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d,
                                       float(sigma), g.data_ptr() if g.numel() else None,
                                       int(g.numel()), buf.data_ptr(), na, flags,
                                       float(diag_shift), st), "qmlg_sargan_kernel")
        return buf.T
    if kind not in ("gaussian", "laplacian"):
        raise ValueError("unknown kernel kind %r" % (kind,))
    fn = lib().qmlg_gaussian_kernel if kind == "gaussian" else lib().qmlg_laplacian_kernel
    check(fn(A.data_ptr(), lda, na, B.data_ptr(), ldb, nb, d, float(sigma), buf.data_ptr(), na,
             flags, float(diag_shift), st), "qmlg_%s_kernel" % kind)
    return buf.T


def gaussian_kernel(A, B, sigma, **kw):
    return kernel_matrix("gaussian", A, B, sigma, **kw)


def laplacian_kernel(A, B, sigma, **kw):
    return kernel_matrix("laplacian", A, B, sigma, **kw)


# ------------------------------------------------------------------ predict --

def predict(kind: str, Xtrain: torch.Tensor, Xtest: torch.Tensor, sigma: float,
            alpha: torch.Tensor, out: Optional[torch.Tensor] = None,
            emulated: bool = False) -> torch.Tensor:
    """yhat = K(Xtest, Xtrain) alpha without materialising the kernel matrix.
    emulated=True uses the fast exact paths: the tensor-core contraction for the
    Gaussian, 64-bit fixed-point L1 sums for the Laplacian."""
    _require_cuda(Xtrain, Xtest, alpha)
    Xtrain, ldtr = _rows(Xtrain)
    Xtest, ldte = _rows(Xtest)
    alpha = alpha.contiguous()
    ntr, nte, d = Xtrain.shape[0], Xtest.shape[0], Xtrain.shape[1]
    if out is None:
        out = torch.empty(nte, dtype=torch.float64, device=Xtrain.device)
    if emulated and kind == "gaussian":
        ws_bytes = lib().qmlg_predict_emulated_workspace_size(ntr, nte, d)
        ws = workspaces.get(ws_bytes, Xtrain.device)
        check(lib().qmlg_predict_emulated(Xtrain.data_ptr(), ldtr, ntr, Xtest.data_ptr(), ldte, nte,
                                          d, float(sigma), alpha.data_ptr(), out.data_ptr(),
                                          ws.data_ptr(), ws.numel(), _stream(Xtrain.device)),
              "qmlg_predict_emulated")
        return out
    if emulated and kind == "laplacian":
        ws_bytes = lib().qmlg_predict_laplacian_fixed_workspace_size(ntr, nte, d)
        ws = workspaces.get(ws_bytes, Xtrain.device)
        check(lib().qmlg_predict_laplacian_fixed(Xtrain.data_ptr(), ldtr, ntr, Xtest.data_ptr(), ldte,
                                                 nte, d, float(sigma), alpha.data_ptr(),
                                                 out.data_ptr(), ws.data_ptr(), ws.numel(),
                                                 _stream(Xtrain.device)),
              "qmlg_predict_laplacian_fixed")
        return out
    ws_bytes = lib().qmlg_predict_workspace_size(ntr, nte)
    ws = workspaces.get(ws_bytes, Xtrain.device)
    check(lib().qmlg_predict_fused(_KINDS[kind], Xtrain.data_ptr(), ldtr, ntr, Xtest.data_ptr(),
                                   ldte, nte, d, float(sigma), alpha.data_ptr(), out.data_ptr(),
                                   ws.data_ptr(), ws.numel(), _stream(Xtrain.device)),
          "qmlg_predict_fused")
    return out


def predict_async(Xtrain: torch.Tensor, Xtest: torch.Tensor, sigma: float, alpha: torch.Tensor,
                  flag: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Gaussian prediction on the tensor cores with no host synchronisation
    (qmlg_predict_emulated_async).  flag: a zeroed int32 CUDA tensor of one element;
    nonzero after the stream completes means recompute with predict(...)."""
    _require_cuda(Xtrain, Xtest, alpha, flag)
    Xtrain, ldtr = _rows(Xtrain)
    Xtest, ldte = _rows(Xtest)
    alpha = alpha.contiguous()
    ntr, nte, d = Xtrain.shape[0], Xtest.shape[0], Xtrain.shape[1]
    if out is None:
        out = torch.empty(nte, dtype=torch.float64, device=Xtrain.device)
    ws_bytes = lib().qmlg_predict_emulated_workspace_size(ntr, nte, d)
    ws = workspaces.get(ws_bytes, Xtrain.device)
    check(lib().qmlg_predict_emulated_async(Xtrain.data_ptr(), ldtr, ntr, Xtest.data_ptr(), ldte,
                                            nte, d, float(sigma), alpha.data_ptr(), out.data_ptr(),
                                            flag.data_ptr(), ws.data_ptr(), ws.numel(),
                                            _stream(Xtrain.device)),
          "qmlg_predict_emulated_async")
    return out


def predict_laplacian_async(Xtrain: torch.Tensor, Xtest: torch.Tensor, sigma: float,
                            alpha: torch.Tensor, flag: Optional[torch.Tensor] = None,
                            out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Laplacian prediction with fixed-point L1 sums and no host synchronisation
    (qmlg_predict_laplacian_fixed_async).  The result is always complete; flag (a
    zeroed int32 CUDA tensor, optional) receives 8 when the FP64 kernel produced it
    because the fixed-point bound was not met."""
    _require_cuda(Xtrain, Xtest, alpha)
    Xtrain, ldtr = _rows(Xtrain)
    Xtest, ldte = _rows(Xtest)
    alpha = alpha.contiguous()
    ntr, nte, d = Xtrain.shape[0], Xtest.shape[0], Xtrain.shape[1]
    if out is None:
        out = torch.empty(nte, dtype=torch.float64, device=Xtrain.device)
    ws_bytes = lib().qmlg_predict_laplacian_fixed_workspace_size(ntr, nte, d)
    ws = workspaces.get(ws_bytes, Xtrain.device)
    check(lib().qmlg_predict_laplacian_fixed_async(
        Xtrain.data_ptr(), ldtr, ntr, Xtest.data_ptr(), ldte, nte, d, float(sigma),
        alpha.data_ptr(), out.data_ptr(), flag.data_ptr() if flag is not None else None,
        ws.data_ptr(), ws.numel(), _stream(Xtrain.device)), "qmlg_predict_laplacian_fixed_async")
    return out


def predict_gemv(Ks: torch.Tensor, alpha: torch.Tensor) -> torch.Tensor:
    """yhat = Ks^T alpha for a Fortran-ordered Ks (ntrain, ntest) (np.dot(Ks.T, alpha))."""
    _require_cuda(Ks, alpha)
    ntr, nte = Ks.shape
    if Ks.stride(0) != 1:
        Ks = Ks.T.contiguous().T
    ldk = max(Ks.stride(1), ntr)
    out = torch.empty(nte, dtype=torch.float64, device=Ks.device)
    check(lib().qmlg_predict_gemv(Ks.data_ptr(), ldk, ntr, nte, alpha.contiguous().data_ptr(),
                                  out.data_ptr(), _stream(Ks.device)), "qmlg_predict_gemv")
    return out


# -------------------------------------------------------------------- solve --

def _colmajor(A: torch.Tensor) -> Tuple[torch.Tensor, int]:
    """Pointer view of A as a column-major matrix: Fortran-ordered tensors are used
    as they are; a C-ordered tensor is its own transpose in column-major terms
    (identical for the symmetric matrices KRR solves)."""
    if A.dim() != 2 or A.shape[0] != A.shape[1] or A.dtype != torch.float64:
        raise ValueError("expected a square float64 matrix")
    n = A.shape[0]
    if A.stride(0) == 1 and A.stride(1) >= n:
        return A, A.stride(1)
    if A.stride(1) == 1 and A.stride(0) >= n:
        return A, A.stride(0)
    raise ValueError("A must be row- or column-contiguous")


def solve(A: torch.Tensor, y: torch.Tensor, lam: float = 0.0, precision: str = "mixed",
          max_outer: int = 10, tol: float = 1e-14, allow_fallback: bool = True,
          raise_on_info: bool = True, slices: int = 0):
    """Solve (A + lam I) x = y on the GPU.  Returns (x, report dict).

    precision "fp64": blocked FP64 Cholesky in place (A's upper triangle in
    column-major terms is overwritten, like dpotrf("U")), then dpotrs and, when
    max_outer > 0, refinement with the exactly summed residual.  precision "mixed":
    the same factor with its trailing updates emulated on the bf16 tensor cores
    (`slices` digit planes, 4..8, 0 = 8), refined in FP64 with the exact residual;
    falls back to the plain FP64 factor when the refinement stalls.  The other
    triangle of A is never written (after a fallback the factorised triangle holds
    the FP64 factor).
    """
    _require_cuda(A, y)
    if precision not in _PRECISIONS:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    Acm, lda = _colmajor(A)
    n = Acm.shape[0]
    if y.shape != (n,):
        raise ValueError("expected matrix and vector of same stride size")
    y = y.contiguous()
    x = torch.empty_like(y)
    p = _PRECISIONS[precision]
    ws_bytes = lib().qmlg_solve_workspace_size(n, p)
    ws = workspaces.get(ws_bytes, A.device)
    opts = QmlgRefineOpts(int(max_outer), 0, float(tol), 0.0, 1 if allow_fallback else 0,
                          int(slices))
    rep = QmlgSolveReport()
    st = lib().qmlg_solve(Acm.data_ptr(), n, lda, y.data_ptr(), x.data_ptr(), float(lam), p,
                          ctypes.byref(opts), ctypes.byref(rep), ws.data_ptr(), ws.numel(),
                          _stream(A.device))
    if st < 0 and st != _lib.QMLG_E_NOT_CONVERGED:
        check(st, "qmlg_solve")
    report = rep.as_dict()
    report["status"] = st
    if st > 0 and raise_on_info:
        raise torch.linalg.LinAlgError(
            "the %d-th leading minor is not positive definite" % st)
    return x, report


def cholesky(A: torch.Tensor, lam: float = 0.0, precision: str = "fp64") -> int:
    """In-place Cholesky with dpotrf("U") semantics; returns LAPACK's info.
    precision "mixed" emulates the trailing updates on the bf16 tensor cores."""
    _require_cuda(A)
    Acm, lda = _colmajor(A)
    n = Acm.shape[0]
    if precision == "mixed":
        size_fn, fn, name = (lib().qmlg_cholesky_mixed_workspace_size, lib().qmlg_cholesky_mixed,
                             "qmlg_cholesky_mixed")
    else:
        size_fn, fn, name = (lib().qmlg_cholesky_workspace_size, lib().qmlg_cholesky,
                             "qmlg_cholesky")
    ws_bytes = size_fn(n)
    ws = workspaces.get(ws_bytes, A.device)
    return check(fn(Acm.data_ptr(), n, lda, float(lam), ws.data_ptr(), ws.numel(),
                    _stream(A.device)), name)


def syrk_emulated(C: torch.Tensor, P: torch.Tensor) -> None:
    """C <- C - P P^T on C's row-major lower triangle, emulated FP64 on the tensor
    cores (the trailing update of the mixed factorisation).  C (n, n) row-major,
    P (n, k) row-major, k <= 512."""
    _require_cuda(C, P)
    n, k = P.shape
    if C.shape != (n, n) or C.stride(1) != 1 or P.stride(1) != 1:
        raise ValueError("C (n, n) and P (n, k) must be row-major")
    ws_bytes = lib().qmlg_syrk_emulated_workspace_size(n, k)
    ws = workspaces.get(ws_bytes, C.device)
    check(lib().qmlg_syrk_emulated(C.data_ptr(), C.stride(0), n, P.data_ptr(), P.stride(0), k,
                                   ws.data_ptr(), ws.numel(), _stream(C.device)),
          "qmlg_syrk_emulated")


def cho_invert(A: torch.Tensor, precision: str = "fp64"):
    """A^-1 of a symmetric positive-definite A (its column-major lower triangle is
    read, like dpotrf("L")).  Returns (Ainv, info): Ainv a Fortran-ordered (n, n)
    float64 view, info LAPACK's (0 = ok)."""
    _require_cuda(A)
    if precision not in _PRECISIONS:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    Acm, lda = _colmajor(A)
    n = Acm.shape[0]
    p = _PRECISIONS[precision]
    out = torch.empty((n, n), dtype=torch.float64, device=A.device)  # rows = columns of Ainv
    ws = workspaces.get(lib().qmlg_cho_invert_workspace_size(n, p), A.device)
    st = lib().qmlg_cho_invert(Acm.data_ptr(), n, lda, out.data_ptr(), n, p, ws.data_ptr(),
                               ws.numel(), _stream(A.device))
    if st < 0:
        check(st, "qmlg_cho_invert")
    return out.T, st


def bkf_solve(A: torch.Tensor, y: torch.Tensor):
    """x with A x = y by Bunch-Kaufman pivoting (A's column-major lower triangle is
    read).  Returns (x, info), info LAPACK's (0 = ok)."""
    _require_cuda(A, y)
    Acm, lda = _colmajor(A)
    n = Acm.shape[0]
    if y.shape != (n,):
        raise ValueError("expected matrix and vector of same stride size")
    y = y.contiguous()
    x = torch.empty_like(y)
    ws = workspaces.get(lib().qmlg_bkf_solve_workspace_size(n), A.device)
    st = lib().qmlg_bkf_solve(Acm.data_ptr(), n, lda, y.data_ptr(), x.data_ptr(), ws.data_ptr(),
                              ws.numel(), _stream(A.device))
    if st < 0:
        check(st, "qmlg_bkf_solve")
    return x, st


def bkf_invert(A: torch.Tensor):
    """A^-1 by Bunch-Kaufman pivoting.  Returns (Ainv, info), Ainv a Fortran-ordered
    (n, n) float64 view."""
    _require_cuda(A)
    Acm, lda = _colmajor(A)
    n = Acm.shape[0]
    out = torch.empty((n, n), dtype=torch.float64, device=A.device)
    ws = workspaces.get(lib().qmlg_bkf_invert_workspace_size(n), A.device)
    st = lib().qmlg_bkf_invert(Acm.data_ptr(), n, lda, out.data_ptr(), n, ws.data_ptr(),
                               ws.numel(), _stream(A.device))
    if st < 0:
        check(st, "qmlg_bkf_invert")
    return out.T, st


def cholesky_solve_factored(U: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    """dpotrs("U", nrhs=1) with a factor from cholesky()."""
    _require_cuda(U, y)
    Ucm, lda = _colmajor(U)
    n = Ucm.shape[0]
    y = y.contiguous()
    x = torch.empty_like(y)
    check(lib().qmlg_cholesky_solve_factored(Ucm.data_ptr(), n, lda, y.data_ptr(), x.data_ptr(),
                                             _stream(U.device)), "qmlg_cholesky_solve_factored")
    return x


def residual_dd(A: torch.Tensor, diag: torch.Tensor, lam: float, x: torch.Tensor,
                y: torch.Tensor) -> torch.Tensor:
    """y - (A + lam I) x summed exactly and rounded once, using A's untouched
    triangle and diag."""
    _require_cuda(A, diag, x, y)
    Acm, lda = _colmajor(A)
    n = Acm.shape[0]
    r = torch.empty_like(y)
    ws_bytes = lib().qmlg_residual_workspace_size(n)
    ws = workspaces.get(ws_bytes, A.device)
    check(lib().qmlg_residual_dd(Acm.data_ptr(), n, lda, diag.contiguous().data_ptr(), float(lam),
                                 x.contiguous().data_ptr(), y.contiguous().data_ptr(),
                                 r.data_ptr(), ws.data_ptr(), ws.numel(), _stream(A.device)),
          "qmlg_residual_dd")
    return r
