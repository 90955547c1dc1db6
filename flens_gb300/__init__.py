"""flens_gb300 -- GB300-native dense GEMM / TRSM / LU behind FLENS's interfaces.

The product is the C-ABI shared library ``libflens_gb300.so`` (CUDA for
sm_103a, declared in ``include/flens_gb300.h``).  This module is a thin ctypes
binding over that library, used by the tests and the benchmark and by Python
callers:

* ``lib()`` -- the loaded ``ctypes.CDLL`` (raises if the library is missing:
  there is no CPU fallback).
* Fortran-ABI wrappers on host numpy arrays (column-major): :func:`dgemm`,
  :func:`dtrsm`, :func:`dgetrf`, :func:`dgetrs`, :func:`dgesv`.  They call the
  exported ``dgemm_``, ``dtrsm_``, ... exactly as a Fortran or C caller would.
* Device wrappers on torch CUDA tensors (column-major = ``tensor.t()`` of a
  contiguous row-major tensor, or any tensor with stride(0)==1):
  :func:`dgemm_dev`, :func:`dtrsm_dev`, :func:`dgetrf_dev`, :func:`dgetrs_dev`,
  :func:`dgesv_dev`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libflens_gb300.so")

ERR_CUDA = -1001
ERR_TIMEOUT = -1002
ERR_NO_DEVICE = -1003
ERR_ALLOC = -1004
ERR_UNSUPPORTED = -1005
ERR_NOT_CONVERGED = -1006

_lib = None
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_c = ctypes.c_char
_i = ctypes.c_int
_d = ctypes.c_double
_v = ctypes.c_void_p


class FlensGB300Error(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().flens_gb300_last_error().decode(errors="replace")
        super().__init__(f"{where} returned {code}: {msg}")
        self.code = code


def build_library() -> str:
    """Compile libflens_gb300.so (nvcc, sm_103a); see flens_gb300/build.py."""
    from . import build as _b
    return _b.build()


def lib() -> ctypes.CDLL:
    """Load libflens_gb300.so (building it first if only the sources exist)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (nvcc for sm_103a)")
    L = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    cp = ctypes.c_char_p
    L.dgemm_.argtypes = [cp, cp, _ip, _ip, _ip, _dp, _dp, _ip, _dp, _ip, _dp, _dp, _ip]
    L.dgemm_.restype = None
    L.dtrsm_.argtypes = [cp, cp, cp, cp, _ip, _ip, _dp, _dp, _ip, _dp, _ip]
    L.dtrsm_.restype = None
    L.dgetrf_.argtypes = [_ip, _ip, _dp, _ip, _ip, _ip]
    L.dgetrf_.restype = None
    L.dgetrs_.argtypes = [cp, _ip, _ip, _dp, _ip, _ip, _dp, _ip, _ip]
    L.dgetrs_.restype = None
    L.dgesv_.argtypes = [_ip, _ip, _dp, _ip, _ip, _dp, _ip, _ip]
    L.dgesv_.restype = None
    L.dsyrk_.argtypes = [cp, cp, _ip, _ip, _dp, _dp, _ip, _dp, _dp, _ip]
    L.dsyrk_.restype = None
    L.dpotrf_.argtypes = [cp, _ip, _dp, _ip, _ip]
    L.dpotrf_.restype = None
    L.dpotrs_.argtypes = [cp, _ip, _ip, _dp, _ip, _dp, _ip, _ip]
    L.dpotrs_.restype = None
    L.dposv_.argtypes = [cp, _ip, _ip, _dp, _ip, _dp, _ip, _ip]
    L.dposv_.restype = None
    L.dtrmm_.argtypes = [cp, cp, cp, cp, _ip, _ip, _dp, _dp, _ip, _dp, _ip]
    L.dtrmm_.restype = None
    L.dsymm_.argtypes = [cp, cp, _ip, _ip, _dp, _dp, _ip, _dp, _ip, _dp, _dp, _ip]
    L.dsymm_.restype = None
    L.dsyr2k_.argtypes = [cp, cp, _ip, _ip, _dp, _dp, _ip, _dp, _ip, _dp, _dp, _ip]
    L.dsyr2k_.restype = None
    L.dtrtri_.argtypes = [cp, cp, _ip, _dp, _ip, _ip]
    L.dtrtri_.restype = None
    L.dgetri_.argtypes = [_ip, _dp, _ip, _ip, _dp, _ip, _ip]
    L.dgetri_.restype = None
    L.dgerfs_.argtypes = [cp, _ip, _ip, _dp, _ip, _dp, _ip, _ip, _dp, _ip, _dp, _ip, _dp, _dp, _dp,
                          _ip, _ip]
    L.dgerfs_.restype = None
    L.dgecon_.argtypes = [cp, _ip, _dp, _ip, _dp, _dp, _dp, _ip, _ip]
    L.dgecon_.restype = None
    L.dgeequ_.argtypes = [_ip, _ip, _dp, _ip, _dp, _dp, _dp, _dp, _dp, _ip]
    L.dgeequ_.restype = None
    L.dlaqge_.argtypes = [_ip, _ip, _dp, _ip, _dp, _dp, _dp, _dp, _dp, cp]
    L.dlaqge_.restype = None
    L.dgesvx_.argtypes = [cp, cp, _ip, _ip, _dp, _ip, _dp, _ip, _ip, cp, _dp, _dp, _dp, _ip, _dp,
                          _ip, _dp, _dp, _dp, _dp, _ip, _ip]
    L.dgesvx_.restype = None
    L.flens_gb300_dgecon.argtypes = [_c, _i, _v, _i, _d, _dp, _v]
    L.flens_gb300_dgerfs.argtypes = [_c, _i, _i, _v, _i, _v, _i, _v, _v, _i, _v, _i, _dp, _dp, _v]
    L.flens_gb300_dgeequ.argtypes = [_i, _i, _v, _i, _v, _v, _dp, _dp, _dp, _ip, _v]
    L.flens_gb300_dlaqge.argtypes = [_i, _i, _v, _i, _v, _v, _d, _d, _d, ctypes.c_char_p, _v]
    L.flens_gb300_dgesvx.argtypes = [_c, _c, _i, _i, _v, _i, _v, _i, _v, ctypes.c_char_p, _v, _v, _v,
                                     _i, _v, _i, _dp, _dp, _dp, _dp, _ip, _v]
    L.flens_gb300_dtrtri.argtypes = [_c, _c, _i, _v, _i, _v, _v]
    L.flens_gb300_dgetri.argtypes = [_i, _v, _i, _v, _v, _v]
    L.flens_gb300_dtrmm.argtypes = [_c, _c, _c, _c, _i, _i, _d, _v, _i, _v, _i, _v]
    L.flens_gb300_dsymm.argtypes = [_c, _c, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _v]
    L.flens_gb300_dsyr2k.argtypes = [_c, _c, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _v]
    L.flens_gb300_dsyrk.argtypes = [_c, _c, _i, _i, _d, _v, _i, _d, _v, _i, _v]
    L.flens_gb300_dpotrf.argtypes = [_c, _i, _v, _i, _v, _v]
    L.flens_gb300_dpotrs.argtypes = [_c, _i, _i, _v, _i, _v, _i, _v]
    L.flens_gb300_dposv.argtypes = [_c, _i, _i, _v, _i, _v, _i, _v, _v]
    L.flens_gb300_dgemm.argtypes = [_c, _c, _i, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _v]
    L.flens_gb300_dtrsm.argtypes = [_c, _c, _c, _c, _i, _i, _d, _v, _i, _v, _i, _v]
    L.flens_gb300_dgetrf.argtypes = [_i, _i, _v, _i, _v, _v, _v]
    L.flens_gb300_dgetrf_split.argtypes = [_i, _i, _v, _i, _v, _v, _i, _v]
    L.flens_gb300_dgetrs.argtypes = [_c, _i, _i, _v, _i, _v, _v, _i, _v]
    L.flens_gb300_dgesv.argtypes = [_i, _i, _v, _i, _v, _v, _i, _v, _v]
    L.flens_gb300_sync.argtypes = [_v]
    L.flens_gb300_dgetrs_noalloc.argtypes = [_c, _i, _i, _v, _i, _v, _v, _i, _v]
    L.flens_gb300_dgetrs_noalloc.restype = _i
    L.flens_gb300_dgemm_split.argtypes = [_c, _c, _i, _i, _i, _d, _v, _i, _v, _i, _d, _v, _i, _i,
                                          ctypes.POINTER(ctypes.c_int), _v]
    L.flens_gb300_dgemm_split.restype = _i
    for f in ("flens_gb300_dgemm", "flens_gb300_dtrsm", "flens_gb300_dgetrf", "flens_gb300_dgetrf_split",
              "flens_gb300_dgetrs", "flens_gb300_dgesv", "flens_gb300_sync",
              "flens_gb300_dsyrk", "flens_gb300_dpotrf", "flens_gb300_dpotrs",
              "flens_gb300_dposv", "flens_gb300_dtrmm", "flens_gb300_dsymm",
              "flens_gb300_dsyr2k", "flens_gb300_dtrtri", "flens_gb300_dgetri",
              "flens_gb300_dgecon", "flens_gb300_dgerfs", "flens_gb300_dgeequ",
              "flens_gb300_dlaqge", "flens_gb300_dgesvx"):
        getattr(L, f).restype = _i
    L.flens_gb300_last_error.restype = ctypes.c_char_p
    L.flens_gb300_last_error.argtypes = []
    L.flens_gb300_xerbla_calls.restype = _i
    L.flens_gb300_xerbla_info.restype = _i
    L.flens_gb300_xerbla_name.restype = ctypes.c_char_p
    L.flens_gb300_version.restype = _i
    L.flens_gb300_launch_count.restype = ctypes.c_longlong
    L.flens_gb300_launch_count.argtypes = []
    L.flens_gb300_timing_enable.argtypes = [_i]
    L.flens_gb300_timing_enable.restype = None
    L.flens_gb300_timing_read.argtypes = [_i, _dp, ctypes.POINTER(ctypes.c_longlong), _dp, _dp]
    L.flens_gb300_timing_read.restype = _i
    L.flens_gb300_family_name.argtypes = [_i]
    L.flens_gb300_family_name.restype = ctypes.c_char_p
    _lib = L
    return L


def last_error() -> str:
    return lib().flens_gb300_last_error().decode(errors="replace")


# ------------------------------------------------------ instrumentation ---
N_FAMILIES = 12


def launch_count() -> int:
    """Kernel launches issued by the library since it was loaded."""
    return int(lib().flens_gb300_launch_count())


def timing_enable(on: bool = True) -> None:
    """Per-launch CUDA-event timing on the launching stream (clears totals)."""
    lib().flens_gb300_timing_enable(1 if on else 0)


def timing_read() -> dict:
    """{family: {ms, launches, flops, bytes}} since timing_enable (synchronises)."""
    out = {}
    for f in range(N_FAMILIES):
        ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        cnt = ctypes.c_longlong()
        lib().flens_gb300_timing_read(f, ctypes.byref(ms), ctypes.byref(cnt), ctypes.byref(fl),
                                      ctypes.byref(by))
        if cnt.value:
            name = lib().flens_gb300_family_name(f).decode()
            out[name] = {"ms": ms.value, "launches": cnt.value, "flops": fl.value,
                         "bytes": by.value}
    return out


# ---------------------------------------------------------- host (numpy) ---
def _ref(v, t):
    return ctypes.byref(t(v))


def _fd(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.f_contiguous:
        raise ValueError("expected a Fortran-ordered float64 array")
    return a.ctypes.data_as(_dp)


def dgemm(transA: str, transB: str, alpha: float, A: np.ndarray, B: np.ndarray,
          beta: float, C: np.ndarray) -> np.ndarray:
    """C <- beta*C + alpha*op(A)*op(B) through dgemm_ (in place on C)."""
    m, n = C.shape
    k = A.shape[1] if transA.upper() == "N" else A.shape[0]
    lib().dgemm_(transA.encode(), transB.encode(), _ref(m, _i), _ref(n, _i), _ref(k, _i),
                 _ref(alpha, _d), _fd(A), _ref(max(1, A.shape[0]), _i), _fd(B),
                 _ref(max(1, B.shape[0]), _i), _ref(beta, _d), _fd(C), _ref(max(1, m), _i))
    return C


def dtrsm(side: str, uplo: str, transA: str, diag: str, alpha: float, A: np.ndarray,
          B: np.ndarray) -> np.ndarray:
    m, n = B.shape
    lib().dtrsm_(side.encode(), uplo.encode(), transA.encode(), diag.encode(),
                 _ref(m, _i), _ref(n, _i), _ref(alpha, _d), _fd(A),
                 _ref(max(1, A.shape[0]), _i), _fd(B), _ref(max(1, m), _i))
    return B


def dgetrf(A: np.ndarray):
    """In-place LU through dgetrf_; returns (ipiv 1-based int32, info)."""
    m, n = A.shape
    piv = np.zeros(max(1, min(m, n)), dtype=np.int32)
    info = ctypes.c_int(0)
    lib().dgetrf_(_ref(m, _i), _ref(n, _i), _fd(A), _ref(max(1, m), _i),
                  piv.ctypes.data_as(_ip), ctypes.byref(info))
    return piv[: min(m, n)], info.value


def dgetrs(trans: str, LU: np.ndarray, ipiv: np.ndarray, B: np.ndarray):
    n = LU.shape[0]
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    info = ctypes.c_int(0)
    lib().dgetrs_(trans.encode(), _ref(n, _i), _ref(B.shape[1], _i), _fd(LU),
                  _ref(max(1, n), _i), ipiv.ctypes.data_as(_ip), _fd(B),
                  _ref(max(1, n), _i), ctypes.byref(info))
    return B, info.value


def dgesv(A: np.ndarray, B: np.ndarray):
    n = A.shape[0]
    piv = np.zeros(max(1, n), dtype=np.int32)
    info = ctypes.c_int(0)
    lib().dgesv_(_ref(n, _i), _ref(B.shape[1], _i), _fd(A), _ref(max(1, n), _i),
                 piv.ctypes.data_as(_ip), _fd(B), _ref(max(1, n), _i), ctypes.byref(info))
    return piv[:n], info.value


def dsyrk(uplo: str, trans: str, alpha: float, A: np.ndarray, beta: float, C: np.ndarray):
    n = C.shape[0]
    k = A.shape[1] if trans.upper() == "N" else A.shape[0]
    lib().dsyrk_(uplo.encode(), trans.encode(), _ref(n, _i), _ref(k, _i), _ref(alpha, _d), _fd(A),
                 _ref(max(1, A.shape[0]), _i), _ref(beta, _d), _fd(C), _ref(max(1, n), _i))
    return C


def dtrmm(side: str, uplo: str, transA: str, diag: str, alpha: float, A: np.ndarray,
          B: np.ndarray) -> np.ndarray:
    m, n = B.shape
    lib().dtrmm_(side.encode(), uplo.encode(), transA.encode(), diag.encode(), _ref(m, _i),
                 _ref(n, _i), _ref(alpha, _d), _fd(A), _ref(max(1, A.shape[0]), _i), _fd(B),
                 _ref(max(1, m), _i))
    return B


def dsymm(side: str, uplo: str, alpha: float, A: np.ndarray, B: np.ndarray, beta: float,
          C: np.ndarray) -> np.ndarray:
    m, n = C.shape
    lib().dsymm_(side.encode(), uplo.encode(), _ref(m, _i), _ref(n, _i), _ref(alpha, _d), _fd(A),
                 _ref(max(1, A.shape[0]), _i), _fd(B), _ref(max(1, m), _i), _ref(beta, _d), _fd(C),
                 _ref(max(1, m), _i))
    return C


def dsyr2k(uplo: str, trans: str, alpha: float, A: np.ndarray, B: np.ndarray, beta: float,
           C: np.ndarray) -> np.ndarray:
    n = C.shape[0]
    k = A.shape[1] if trans.upper() == "N" else A.shape[0]
    lib().dsyr2k_(uplo.encode(), trans.encode(), _ref(n, _i), _ref(k, _i), _ref(alpha, _d), _fd(A),
                  _ref(max(1, A.shape[0]), _i), _fd(B), _ref(max(1, B.shape[0]), _i),
                  _ref(beta, _d), _fd(C), _ref(max(1, n), _i))
    return C


def dtrtri(uplo: str, diag: str, A: np.ndarray) -> int:
    """In-place triangular inverse through dtrtri_; returns info."""
    n = A.shape[0]
    info = ctypes.c_int(0)
    lib().dtrtri_(uplo.encode(), diag.encode(), _ref(n, _i), _fd(A), _ref(max(1, n), _i),
                  ctypes.byref(info))
    return info.value


def dgetri(A: np.ndarray, ipiv: np.ndarray) -> int:
    """In-place inverse from dgetrf_'s factors through dgetri_; returns info."""
    n = A.shape[0]
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    work = np.zeros(max(1, n))
    info = ctypes.c_int(0)
    lib().dgetri_(_ref(n, _i), _fd(A), _ref(max(1, n), _i), ipiv.ctypes.data_as(_ip),
                  work.ctypes.data_as(_dp), _ref(work.size, _i), ctypes.byref(info))
    return info.value


def dgecon(norm: str, LU: np.ndarray, anorm: float):
    """Reciprocal condition number estimate from dgetrf_'s factors: (rcond, info)."""
    n = LU.shape[0]
    rc, info = ctypes.c_double(0.0), ctypes.c_int(0)
    work, iwork = np.zeros(max(1, 4 * n)), np.zeros(max(1, n), dtype=np.int32)
    lib().dgecon_(norm.encode(), _ref(n, _i), _fd(LU), _ref(max(1, n), _i), _ref(anorm, _d),
                  ctypes.byref(rc), work.ctypes.data_as(_dp), iwork.ctypes.data_as(_ip),
                  ctypes.byref(info))
    return rc.value, info.value


def dgerfs(trans: str, A: np.ndarray, LU: np.ndarray, ipiv: np.ndarray, B: np.ndarray,
           X: np.ndarray):
    """Refine X in place through dgerfs_; returns (ferr, berr, info)."""
    n, k = B.shape
    ferr, berr = np.zeros(max(1, k)), np.zeros(max(1, k))
    work, iwork = np.zeros(max(1, 3 * n)), np.zeros(max(1, n), dtype=np.int32)
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
    info = ctypes.c_int(0)
    lib().dgerfs_(trans.encode(), _ref(n, _i), _ref(k, _i), _fd(A), _ref(max(1, n), _i), _fd(LU),
                  _ref(max(1, n), _i), ipiv.ctypes.data_as(_ip), _fd(B), _ref(max(1, n), _i), _fd(X),
                  _ref(max(1, n), _i), ferr.ctypes.data_as(_dp), berr.ctypes.data_as(_dp),
                  work.ctypes.data_as(_dp), iwork.ctypes.data_as(_ip), ctypes.byref(info))
    return ferr[:k], berr[:k], info.value


def dgeequ(A: np.ndarray):
    m, n = A.shape
    r, c = np.zeros(max(1, m)), np.zeros(max(1, n))
    rc, cc, am, info = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    lib().dgeequ_(_ref(m, _i), _ref(n, _i), _fd(A), _ref(max(1, m), _i), r.ctypes.data_as(_dp),
                  c.ctypes.data_as(_dp), ctypes.byref(rc), ctypes.byref(cc), ctypes.byref(am),
                  ctypes.byref(info))
    return r[:m], c[:n], rc.value, cc.value, am.value, info.value


def dlaqge(A: np.ndarray, r, c, rowcnd: float, colcnd: float, amax: float) -> str:
    m, n = A.shape
    r = np.ascontiguousarray(r, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    eq = ctypes.create_string_buffer(b"?", 2)
    lib().dlaqge_(_ref(m, _i), _ref(n, _i), _fd(A), _ref(max(1, m), _i), r.ctypes.data_as(_dp),
                  c.ctypes.data_as(_dp), _ref(rowcnd, _d), _ref(colcnd, _d), _ref(amax, _d), eq)
    return eq.value.decode()


def dgesvx(fact: str, trans: str, A: np.ndarray, AF: np.ndarray, ipiv: np.ndarray, equed: str,
           r: np.ndarray, c: np.ndarray, B: np.ndarray, X: np.ndarray):
    """Expert driver through dgesvx_: (info, equed, rcond, ferr, berr, rpvgrw)."""
    n, k = B.shape
    eq = ctypes.create_string_buffer(equed.encode(), 2)
    rc, info = ctypes.c_double(0.0), ctypes.c_int(0)
    ferr, berr = np.zeros(max(1, k)), np.zeros(max(1, k))
    work, iwork = np.zeros(max(1, 4 * n)), np.zeros(max(1, n), dtype=np.int32)
    lib().dgesvx_(fact.encode(), trans.encode(), _ref(n, _i), _ref(k, _i), _fd(A), _ref(max(1, n), _i),
                  _fd(AF), _ref(max(1, n), _i), ipiv.ctypes.data_as(_ip), eq, r.ctypes.data_as(_dp),
                  c.ctypes.data_as(_dp), _fd(B), _ref(max(1, n), _i), _fd(X), _ref(max(1, n), _i),
                  ctypes.byref(rc), ferr.ctypes.data_as(_dp), berr.ctypes.data_as(_dp),
                  work.ctypes.data_as(_dp), iwork.ctypes.data_as(_ip), ctypes.byref(info))
    return info.value, eq.value.decode(), rc.value, ferr[:k], berr[:k], work[0]


def dpotrf(uplo: str, A: np.ndarray) -> int:
    """In-place Cholesky through dpotrf_; returns info."""
    n = A.shape[0]
    info = ctypes.c_int(0)
    lib().dpotrf_(uplo.encode(), _ref(n, _i), _fd(A), _ref(max(1, n), _i), ctypes.byref(info))
    return info.value


def dpotrs(uplo: str, A: np.ndarray, B: np.ndarray):
    n = A.shape[0]
    info = ctypes.c_int(0)
    lib().dpotrs_(uplo.encode(), _ref(n, _i), _ref(B.shape[1], _i), _fd(A), _ref(max(1, n), _i),
                  _fd(B), _ref(max(1, n), _i), ctypes.byref(info))
    return B, info.value


def dposv(uplo: str, A: np.ndarray, B: np.ndarray) -> int:
    n = A.shape[0]
    info = ctypes.c_int(0)
    lib().dposv_(uplo.encode(), _ref(n, _i), _ref(B.shape[1], _i), _fd(A), _ref(max(1, n), _i),
                 _fd(B), _ref(max(1, n), _i), ctypes.byref(info))
    return info.value


# -------------------------------------------------------- device (torch) ---
def _colmajor(t):
    """(pointer, rows, cols, ld) of a column-major CUDA float64 tensor."""
    if t.dim() == 2 and t.numel() == 0:
        return t.data_ptr(), t.shape[0], t.shape[1], max(1, t.shape[0])
    if t.dim() != 2 or (t.stride(0) != 1 and t.shape[0] != 1):   # a 1-row stride is free
        raise ValueError("expected a 2-D column-major tensor (stride(0) == 1)")
    return t.data_ptr(), t.shape[0], t.shape[1], max(1, t.stride(1), t.shape[0])


def _stream(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _check(code: int, where: str) -> None:
    if code != 0:
        raise FlensGB300Error(code, where)


def colmajor_empty(m: int, n: int, dtype=None, device="cuda"):
    """A column-major (m x n) tensor: storage of an (n x m) row-major one, transposed."""
    import torch
    return torch.empty((n, m), dtype=dtype or torch.float64, device=device).t()


def to_colmajor(t):
    return t.t().contiguous().t()


def dgemm_dev(transA, transB, alpha, A, B, beta, C, stream=None):
    pa, ra, ca, lda = _colmajor(A)
    pb, rb, cb, ldb = _colmajor(B)
    pc, m, n, ldc = _colmajor(C)
    k = ca if transA.upper() == "N" else ra
    _check(lib().flens_gb300_dgemm(transA.encode(), transB.encode(), m, n, k, alpha, pa, lda,
                                   pb, ldb, beta, pc, ldc, _stream(stream)), "flens_gb300_dgemm")
    return C


def dgemm_split_dev(transA, transB, alpha, A, B, beta, C, slices=0, stream=None):
    """FP64-accurate C <- beta*C + alpha*op(A)*op(B) from exact BF16 tensor-core
    products of exponent-aligned slices (device tensors, column-major).
    slices = 0 picks the slice count from the data.  Returns the slice count
    used (-1: the inputs needed the plain FP64 kernel).  Synchronises."""
    pa, ra, ca, lda = _colmajor(A)
    pb, rb, cb, ldb = _colmajor(B)
    pc, m, n, ldc = _colmajor(C)
    k = ca if transA.upper() == "N" else ra
    used = ctypes.c_int(0)
    _check(lib().flens_gb300_dgemm_split(transA.encode(), transB.encode(), m, n, k, alpha, pa, lda,
                                         pb, ldb, beta, pc, ldc, slices, ctypes.byref(used),
                                         _stream(stream)), "flens_gb300_dgemm_split")
    return used.value


def dsyrk_dev(uplo, trans, alpha, A, beta, C, stream=None):
    pa, ra, ca, lda = _colmajor(A)
    pc, n, _, ldc = _colmajor(C)
    k = ca if trans.upper() == "N" else ra
    _check(lib().flens_gb300_dsyrk(uplo.encode(), trans.encode(), n, k, alpha, pa, lda, beta, pc,
                                   ldc, _stream(stream)), "flens_gb300_dsyrk")
    return C


def dpotrf_dev(uplo, A, info, stream=None):
    """In-place Cholesky of a column-major CUDA tensor; info is an int32 CUDA tensor."""
    pa, n, _, lda = _colmajor(A)
    _check(lib().flens_gb300_dpotrf(uplo.encode(), n, pa, lda, info.data_ptr(), _stream(stream)),
           "flens_gb300_dpotrf")
    return A


def dpotrs_dev(uplo, A, B, stream=None):
    pa, n, _, lda = _colmajor(A)
    pb, _, nrhs, ldb = _colmajor(B)
    _check(lib().flens_gb300_dpotrs(uplo.encode(), n, nrhs, pa, lda, pb, ldb, _stream(stream)),
           "flens_gb300_dpotrs")
    return B


def dposv_dev(uplo, A, B, info, stream=None):
    pa, n, _, lda = _colmajor(A)
    pb, _, nrhs, ldb = _colmajor(B)
    _check(lib().flens_gb300_dposv(uplo.encode(), n, nrhs, pa, lda, pb, ldb, info.data_ptr(),
                                   _stream(stream)), "flens_gb300_dposv")
    return B


def dtrsm_dev(side, uplo, transA, diag, alpha, A, B, stream=None):
    pa, ra, ca, lda = _colmajor(A)
    pb, m, n, ldb = _colmajor(B)
    _check(lib().flens_gb300_dtrsm(side.encode(), uplo.encode(), transA.encode(), diag.encode(),
                                   m, n, alpha, pa, lda, pb, ldb, _stream(stream)),
           "flens_gb300_dtrsm")
    return B


def dgetrf_dev(A, ipiv, info, stream=None):
    """In-place LU of a column-major CUDA tensor; ipiv/info are int32 CUDA tensors."""
    pa, m, n, lda = _colmajor(A)
    _check(lib().flens_gb300_dgetrf(m, n, pa, lda, ipiv.data_ptr(), info.data_ptr(),
                                    _stream(stream)), "flens_gb300_dgetrf")
    return A


def dgetrf_split_dev(A, ipiv, info, outer_nb=0, stream=None):
    """FP64-accurate LU of a column-major CUDA tensor with the trailing
    updates on the tensor cores (split GEMM); ipiv/info int32 CUDA tensors."""
    pa, m, n, lda = _colmajor(A)
    _check(lib().flens_gb300_dgetrf_split(m, n, pa, lda, ipiv.data_ptr(), info.data_ptr(), outer_nb,
                                          _stream(stream)), "flens_gb300_dgetrf_split")
    return A


def dgetrs_dev(trans, LU, ipiv, B, stream=None):
    pa, n, _, lda = _colmajor(LU)
    pb, _, nrhs, ldb = _colmajor(B)
    _check(lib().flens_gb300_dgetrs(trans.encode(), n, nrhs, pa, lda, ipiv.data_ptr(), pb, ldb,
                                    _stream(stream)), "flens_gb300_dgetrs")
    return B


def dgesv_dev(A, ipiv, B, info, stream=None):
    pa, n, _, lda = _colmajor(A)
    pb, _, nrhs, ldb = _colmajor(B)
    _check(lib().flens_gb300_dgesv(n, nrhs, pa, lda, ipiv.data_ptr(), pb, ldb, info.data_ptr(),
                                   _stream(stream)), "flens_gb300_dgesv")
    return B


def sync(stream=None) -> None:
    _check(lib().flens_gb300_sync(_stream(stream)), "flens_gb300_sync")
