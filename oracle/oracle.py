"""CPU oracle for the KRR hot path (test infrastructure, never the product).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  It restates the
reference's algorithms:

* ``cm_sorted`` / ``cm_unsorted``: ``qml/frepresentations.f90:52-140`` and
  ``:142-205`` (C restatement in ``qmlg_oracle.c``; ``cm_sorted_numpy`` is an
  independent NumPy restatement used to cross-check the C one);
* ``gaussian_kernel`` / ``laplacian_kernel``: ``qml/fkernels.f90:340-400`` (C, OpenMP);
* ``cho_solve``: ``qml/fcho_solve.f90:23-52`` + ``qml/math.py:60-97``, i.e. LAPACK
  ``dpotrf("U")`` + ``dpotrs("U")``.  LAPACK is third party and not vendored; the
  reference links whatever system LAPACK/MKL is present (no pinned version), here
  the routines come from SciPy's bundled OpenBLAS;
* ``refined_solve``: FP64 Cholesky plus iterative refinement whose residual is
  carried in double-double, giving the solution of (K + lambda I) x = y for the
  given FP64 K to far below FP64 LAPACK's forward error.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libqmlg_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc, OpenMP, no FMA contraction)."""
    src = os.path.join(_HERE, "qmlg_oracle.c")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        lib.oracle_cm_sorted.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, _dp]
        lib.oracle_cm_sorted.restype = ctypes.c_int
        lib.oracle_cm_unsorted.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, _dp]
        lib.oracle_cm_unsorted.restype = ctypes.c_int
        lib.oracle_cm_sorted_batch.argtypes = [_dp, _dp, _i64p, ctypes.c_int, ctypes.c_int, _dp]
        lib.oracle_cm_sorted_batch.restype = ctypes.c_int
        for name in ("oracle_gaussian_kernel", "oracle_laplacian_kernel"):
            fn = getattr(lib, name)
            fn.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp]
            fn.restype = None
        lib.oracle_linear_kernel.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, _dp]
        lib.oracle_linear_kernel.restype = None
        lib.oracle_matern_kernel_l2.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_int, _dp]
        lib.oracle_matern_kernel_l2.restype = None
        lib.oracle_sargan_kernel.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, _dp, ctypes.c_int, _dp]
        lib.oracle_sargan_kernel.restype = None
        _ip = ctypes.POINTER(ctypes.c_int)
        lib.oracle_atomic_cm.argtypes = [_dp, _dp, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, _dp]
        lib.oracle_atomic_cm.restype = ctypes.c_int
        lib.oracle_local_kernels.argtypes = [ctypes.c_int, _dp, _ip, ctypes.c_int, _dp, _ip,
                                             ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp]
        lib.oracle_local_kernels.restype = None
        lib.oracle_residual_dd.argtypes = [_dp, ctypes.c_int, ctypes.c_int64, ctypes.c_double,
                                           _dp, _dp, _dp]
        lib.oracle_residual_dd.restype = None
        lib.oracle_rows_residual_dd.argtypes = [_dp, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                                _dp, _dp, _dp]
        lib.oracle_rows_residual_dd.restype = None
        _lib = lib
    return _lib


def _ptr(a, ctype=_dp):
    return a.ctypes.data_as(ctype)


def cm_sorted(charges, coordinates, size=23):
    """One molecule's row-norm sorted Coulomb matrix, shape (size*(size+1)//2,)."""
    z = np.ascontiguousarray(charges, dtype=np.float64)
    r = np.ascontiguousarray(coordinates, dtype=np.float64)
    out = np.empty(size * (size + 1) // 2)
    if _load().oracle_cm_sorted(_ptr(z), _ptr(r), z.shape[0], size, _ptr(out)) != 0:
        raise ValueError("natoms > size")
    return out


def cm_unsorted(charges, coordinates, size=23):
    z = np.ascontiguousarray(charges, dtype=np.float64)
    r = np.ascontiguousarray(coordinates, dtype=np.float64)
    out = np.empty(size * (size + 1) // 2)
    if _load().oracle_cm_unsorted(_ptr(z), _ptr(r), z.shape[0], size, _ptr(out)) != 0:
        raise ValueError("natoms > size")
    return out


def cm_sorted_batch(charges, coordinates, offsets, size=23):
    z = np.ascontiguousarray(charges, dtype=np.float64)
    r = np.ascontiguousarray(coordinates, dtype=np.float64)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    n_mol = off.shape[0] - 1
    out = np.empty((n_mol, size * (size + 1) // 2))
    if _load().oracle_cm_sorted_batch(_ptr(z), _ptr(r), _ptr(off, _i64p), n_mol, size,
                                      _ptr(out)) != 0:
        raise ValueError("a molecule has more atoms than size")
    return out


def cm_sorted_numpy(charges, coordinates, size=23):
    """Independent NumPy restatement of frepresentations.f90:52-140 (same order of
    operations as the C one, used to cross-check it)."""
    z = np.asarray(charges, dtype=np.float64)
    r = np.asarray(coordinates, dtype=np.float64)
    n = z.shape[0]
    m = np.zeros((n, n))
    for i in range(n):
        m[i, i] = 0.5 * z[i] ** 2.4
        for j in range(i + 1, n):
            d = r[j] - r[i]
            s = d[0] * d[0]
            s = s + d[1] * d[1]
            s = s + d[2] * d[2]
            m[i, j] = m[j, i] = (z[i] * z[j]) / np.sqrt(s)
    rn = np.empty(n)
    for i in range(n):
        acc = m[i, i] * m[i, i]
        for j in range(n):
            if j != i:
                acc = acc + m[i, j] * m[i, j]
        rn[i] = acc
    order = np.empty(n, dtype=np.int64)
    for k in range(n):
        best = int(np.argmin(rn))          # first index of the minimum, like minloc
        order[n - 1 - k] = best
        rn[best] = np.finfo(np.float64).max
    out = np.zeros(size * (size + 1) // 2)
    for a in range(n):
        base = a * (a + 1) // 2
        for b in range(a + 1):
            out[base + b] = m[order[a], order[b]]
    return out


def atomic_cm(charges, coordinates, central=None, size=23, sorting="distance",
              central_cutoff=1e6, central_decay=-1.0, interaction_cutoff=1e6,
              interaction_decay=-1.0):
    """Atomic Coulomb matrices of one molecule, one row per central atom (0-based
    indices, default all), like generate_atomic_coulomb_matrix (qml/representations.py:
    121-230) with sorting "row-norm" or "distance"."""
    z = np.ascontiguousarray(charges, dtype=np.float64)
    r = np.ascontiguousarray(coordinates, dtype=np.float64).reshape(-1, 3)
    if central is None:
        central = np.arange(z.shape[0])
    c = np.ascontiguousarray(central, dtype=np.int32).reshape(-1)
    out = np.zeros((c.shape[0], size * (size + 1) // 2))
    st = _load().oracle_atomic_cm(_ptr(z), _ptr(r), z.shape[0], _ptr(c, ctypes.POINTER(ctypes.c_int)),
                                  c.shape[0], size, 1 if sorting == "row-norm" else 0,
                                  float(central_cutoff), float(central_decay),
                                  float(interaction_cutoff), float(interaction_decay), _ptr(out))
    if st != 0:
        raise ValueError("atomic Coulomb matrix: bad central index or too many atoms within the cutoff")
    return out


def local_kernels(kind, A, B, na, nb, sigmas):
    """get_local_kernels_gaussian / _laplacian (qml/kernels.py:218-299): shape
    (nsigmas, len(na), len(nb))."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    n1 = np.ascontiguousarray(na, dtype=np.int32)
    n2 = np.ascontiguousarray(nb, dtype=np.int32)
    sg = np.ascontiguousarray(sigmas, dtype=np.float64).reshape(-1)
    K = np.zeros((sg.shape[0], n1.shape[0], n2.shape[0]), order="F")
    ip = ctypes.POINTER(ctypes.c_int)
    _load().oracle_local_kernels(0 if kind == "gaussian" else 1, _ptr(A), _ptr(n1, ip), n1.shape[0],
                                 _ptr(B), _ptr(n2, ip), n2.shape[0], A.shape[1], _ptr(sg),
                                 sg.shape[0], _ptr(K))
    return K


def gaussian_kernel(A, B, sigma):
    """K (na, nb) in Fortran order, like qml.kernels.gaussian_kernel."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    K = np.empty((A.shape[0], B.shape[0]), order="F")
    _load().oracle_gaussian_kernel(_ptr(A), A.shape[0], _ptr(B), B.shape[0], A.shape[1],
                                   float(sigma), _ptr(K))
    return K


def laplacian_kernel(A, B, sigma):
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    K = np.empty((A.shape[0], B.shape[0]), order="F")
    _load().oracle_laplacian_kernel(_ptr(A), A.shape[0], _ptr(B), B.shape[0], A.shape[1],
                                    float(sigma), _ptr(K))
    return K


def linear_kernel(A, B):
    """K (na, nb) = A . B^T in Fortran order (qml/fkernels.f90:403-423)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    K = np.empty((A.shape[0], B.shape[0]), order="F")
    _load().oracle_linear_kernel(_ptr(A), A.shape[0], _ptr(B), B.shape[0], A.shape[1], _ptr(K))
    return K


def matern_kernel_l2(A, B, sigma, order):
    """Matern kernel with the L2 distance (qml/fkernels.f90:426-484)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    K = np.empty((A.shape[0], B.shape[0]), order="F")
    _load().oracle_matern_kernel_l2(_ptr(A), A.shape[0], _ptr(B), B.shape[0], A.shape[1],
                                    float(sigma), int(order), _ptr(K))
    return K


def sargan_kernel(A, B, sigma, gammas):
    """Sargan kernel (qml/fkernels.f90:487-531)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    g = np.ascontiguousarray(gammas, dtype=np.float64).reshape(-1)
    K = np.empty((A.shape[0], B.shape[0]), order="F")
    _load().oracle_sargan_kernel(_ptr(A), A.shape[0], _ptr(B), B.shape[0], A.shape[1],
                                 float(sigma), _ptr(g) if g.size else None, int(g.size), _ptr(K))
    return K


def cho_solve(A, y):
    """LAPACK dpotrf("U") + dpotrs("U") on a copy of A (qml/fcho_solve.f90:23-52)."""
    from scipy.linalg import lapack
    a = np.array(A, dtype=np.float64, order="F", copy=True)
    c, info = lapack.dpotrf(a, lower=0, overwrite_a=1, clean=0)
    if info != 0:
        raise np.linalg.LinAlgError("dpotrf info=%d" % info)
    x, info = lapack.dpotrs(c, np.asarray(y, dtype=np.float64), lower=0)
    return x


def cho_invert(A):
    """LAPACK dpotrf("L") + dpotri("L") on a copy (qml/fcho_solve.f90:54-73), the
    lower triangle mirrored to the upper one like qml/math.py:52-56."""
    from scipy.linalg import lapack
    a = np.array(A, dtype=np.float64, order="F", copy=True)
    c, info = lapack.dpotrf(a, lower=1, overwrite_a=1, clean=1)
    if info != 0:
        raise np.linalg.LinAlgError("dpotrf info=%d" % info)
    inv, info = lapack.dpotri(c, lower=1)
    il = np.tril_indices_from(inv)
    inv.T[il] = inv[il]
    return inv


def bkf_solve(A, y):
    """LAPACK dsytrf("L") + dsytrs("L") on a copy (qml/fcho_solve.f90:115-150)."""
    from scipy.linalg import lapack
    a = np.array(A, dtype=np.float64, order="F", copy=True)
    ldu, ipiv, info = lapack.dsytrf(a, lower=1)
    x, info2 = lapack.dsytrs(ldu, ipiv, np.asarray(y, dtype=np.float64), lower=1)
    return x, info


def bkf_invert(A):
    """LAPACK dsytrf("L") + dsytri("L") on a copy (qml/fcho_solve.f90:76-112), the
    lower triangle mirrored like qml/math.py:117-120."""
    from scipy.linalg import lapack
    a = np.array(A, dtype=np.float64, order="F", copy=True)
    ldu, ipiv, info = lapack.dsytrf(a, lower=1)
    inv, info2 = lapack.dsytri(ldu, ipiv, lower=1)
    il = np.tril_indices_from(inv)
    inv.T[il] = inv[il]
    return inv, info


def residual_dd(A, lam, x, y):
    """y - (A + lam I) x with double-double accumulation, rounded to FP64."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    if not A.flags.c_contiguous:
        A = np.ascontiguousarray(A)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    r = np.empty_like(x)
    _load().oracle_residual_dd(_ptr(A), A.shape[0], A.strides[0] // 8, float(lam), _ptr(x),
                               _ptr(y), _ptr(r))
    return r


def rows_residual_dd(A, x, y):
    """y - A x for an (m, n) block of rows, with double-double accumulation."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    if A.ndim != 2 or x.shape != (A.shape[1],) or y.shape != (A.shape[0],):
        raise ValueError("A (m, n), x (n,), y (m,)")
    r = np.empty(A.shape[0])
    _load().oracle_rows_residual_dd(_ptr(A), A.shape[0], A.shape[1], A.strides[0] // 8, _ptr(x),
                                    _ptr(y), _ptr(r))
    return r


def refined_solve(K, y, lam, iters=30, tol=1e-18):
    """Solution of (K + lam I) x = y for the FP64 matrix K, refined with a
    double-double residual until the correction stops shrinking."""
    from scipy.linalg import lapack
    K = np.ascontiguousarray(K, dtype=np.float64)
    n = K.shape[0]
    a = np.array(K, order="F", copy=True)
    a[np.diag_indices(n)] += lam
    c, info = lapack.dpotrf(a, lower=0, overwrite_a=1, clean=0)
    if info != 0:
        raise np.linalg.LinAlgError("dpotrf info=%d" % info)
    x, _ = lapack.dpotrs(c, y, lower=0)
    prev = np.inf
    for _ in range(iters):
        r = residual_dd(K, lam, x, y)
        d, _ = lapack.dpotrs(c, r, lower=0)
        x = x + d
        rel = np.linalg.norm(d) / max(np.linalg.norm(x), 1e-300)
        if rel < tol or rel >= prev:
            break
        prev = rel
    return x


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv))
