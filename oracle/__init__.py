"""Oracle loader -- TEST INFRASTRUCTURE ONLY.

Loads the CPU restatement of FLENS's generic GEMM/TRSM/LU path
(``libflens_oracle.so`` built from ``flens_oracle.c``) and, when it was built
in this checkout, the reference's own Fortran-ABI shims compiled from source
(``_ref/libflens_ref.so``).  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import this package; the product
library never does.

All wrappers take numpy arrays in Fortran (column-major) order and work in
place like the LAPACK routines they mirror.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libflens_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libflens_ref.so")


def _reference_src() -> str:
    """Where the FLENS sources are read from: $FLENS_REFERENCE, else the REF
    default of this directory's Makefile (the recipe that compiles them)."""
    env = os.environ.get("FLENS_REFERENCE")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                if line.split("?=")[0].strip() == "REF" and "?=" in line:
                    return line.split("?=", 1)[1].strip()
    except OSError:
        pass
    return ""


REFERENCE_SRC = _reference_src()

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_double_p = ctypes.POINTER(ctypes.c_double)


def build(with_ref: bool | None = None) -> None:
    """Compile the restatement, and the reference shims if the sources exist."""
    targets = ["port"]
    if with_ref is None:
        with_ref = bool(REFERENCE_SRC) and os.path.isdir(REFERENCE_SRC)
    if with_ref:
        targets.append("ref")
    extra = [f"REF={REFERENCE_SRC}"] if with_ref and REFERENCE_SRC else []
    subprocess.run(["make", "-s", "-j8", "-C", HERE] + targets + extra, check=True)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_c_double_p)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_c_int_p)


def _check_f64(a: np.ndarray) -> None:
    if a.dtype != np.float64 or not a.flags.f_contiguous:
        raise ValueError("expected a Fortran-ordered float64 array")


class Port:
    """ctypes view of the C restatement (oracle_* symbols)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build(with_ref=False)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        c, i, d = ctypes.c_char, ctypes.c_int, ctypes.c_double
        L.oracle_dgemm.argtypes = [c, c, i, i, i, d, _c_double_p, i, _c_double_p, i,
                                   d, _c_double_p, i]
        L.oracle_dtrsm.argtypes = [c, c, c, c, i, i, d, _c_double_p, i, _c_double_p, i]
        L.oracle_idamax.argtypes = [i, _c_double_p, i]
        L.oracle_idamax.restype = i
        L.oracle_dlaswp.argtypes = [i, _c_double_p, i, i, i, _c_int_p, i]
        L.oracle_dgetf2.argtypes = [i, i, _c_double_p, i, _c_int_p]
        L.oracle_dgetf2.restype = i
        L.oracle_dgetrf_nb.argtypes = [i, i, _c_double_p, i, _c_int_p, i]
        L.oracle_dgetrf_nb.restype = i
        L.oracle_dgetrf.argtypes = [i, i, _c_double_p, i, _c_int_p]
        L.oracle_dgetrf.restype = i
        L.oracle_dgetrf_steps.argtypes = [i, i, _c_double_p, i, _c_int_p, i, i]
        L.oracle_dgetrf_steps.restype = i
        L.oracle_dgetrs.argtypes = [c, i, i, _c_double_p, i, _c_int_p, _c_double_p, i]
        L.oracle_dgesv.argtypes = [i, i, _c_double_p, i, _c_int_p, _c_double_p, i]
        L.oracle_dgesv.restype = i
        L.oracle_dsyrk.argtypes = [c, c, i, i, d, _c_double_p, i, d, _c_double_p, i]
        L.oracle_dtrmm.argtypes = [c, c, c, c, i, i, d, _c_double_p, i, _c_double_p, i]
        L.oracle_dsymm.argtypes = [c, c, i, i, d, _c_double_p, i, _c_double_p, i, d,
                                   _c_double_p, i]
        L.oracle_dsyr2k.argtypes = [c, c, i, i, d, _c_double_p, i, _c_double_p, i, d,
                                    _c_double_p, i]
        L.oracle_dpotrf_nb.argtypes = [c, i, _c_double_p, i, i]
        L.oracle_dpotrf_nb.restype = i
        L.oracle_dpotrs.argtypes = [c, i, i, _c_double_p, i, _c_double_p, i]
        L.oracle_dposv.argtypes = [c, i, i, _c_double_p, i, _c_double_p, i]
        L.oracle_dposv.restype = i
        L.oracle_dtrtri_nb.argtypes = [c, c, i, _c_double_p, i, i]
        L.oracle_dtrtri_nb.restype = i
        L.oracle_dgetri.argtypes = [i, _c_double_p, i, _c_int_p]
        L.oracle_dgetri.restype = i
        L.oracle_dlange.argtypes = [c, i, i, _c_double_p, i]
        L.oracle_dlange.restype = d
        L.oracle_dgecon.argtypes = [c, i, _c_double_p, i, d, _c_double_p]
        L.oracle_dgecon.restype = i
        L.oracle_dgerfs.argtypes = [c, i, i, _c_double_p, i, _c_double_p, i, _c_int_p, _c_double_p,
                                    i, _c_double_p, i, _c_double_p, _c_double_p]
        L.oracle_dgerfs.restype = i
        L.oracle_dgeequ.argtypes = [i, i, _c_double_p, i, _c_double_p, _c_double_p, _c_double_p,
                                    _c_double_p, _c_double_p]
        L.oracle_dgeequ.restype = i
        L.oracle_dlaqge.argtypes = [i, i, _c_double_p, i, _c_double_p, _c_double_p, d, d, d]
        L.oracle_dlaqge.restype = c
        L.oracle_dgesvx.argtypes = [c, c, i, i, _c_double_p, i, _c_double_p, i, _c_int_p,
                                    ctypes.c_char_p, _c_double_p, _c_double_p, _c_double_p, i,
                                    _c_double_p, i, _c_double_p, _c_double_p, _c_double_p,
                                    _c_double_p]
        L.oracle_dgesvx.restype = i
        L.oracle_dgetrf_gaps.argtypes = [i, i, _c_double_p, i, _c_int_p, _c_double_p]
        L.oracle_dgetrf_gaps.restype = i
        L.oracle_time_dgetrf_steps.argtypes = [i, i, i, ctypes.c_ulonglong, _c_double_p]
        L.oracle_time_dgetrf_steps.restype = d
        L.oracle_time_dgetrf_step_at.argtypes = [i, i, i, ctypes.c_ulonglong, _c_double_p]
        L.oracle_time_dgetrf_step_at.restype = d
        L.oracle_time_dgemm_rows.argtypes = [i, i, i, i, i, ctypes.c_ulonglong]
        L.oracle_time_dgemm_rows.restype = d

    # -- level 3 ---------------------------------------------------------
    def dgemm(self, transA, transB, alpha, A, B, beta, C):
        _check_f64(A), _check_f64(B), _check_f64(C)
        m, n = C.shape
        k = A.shape[1] if transA.upper() == "N" else A.shape[0]
        self.lib.oracle_dgemm(transA.encode(), transB.encode(), m, n, k, alpha,
                              _dp(A), max(1, A.shape[0]), _dp(B), max(1, B.shape[0]),
                              beta, _dp(C), max(1, m))
        return C

    def dtrsm(self, side, uplo, transA, diag, alpha, A, B):
        _check_f64(A), _check_f64(B)
        m, n = B.shape
        self.lib.oracle_dtrsm(side.encode(), uplo.encode(), transA.encode(),
                              diag.encode(), m, n, alpha, _dp(A), max(1, A.shape[0]),
                              _dp(B), max(1, m))
        return B

    # -- LU ----------------------------------------------------------------
    def idamax(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return self.lib.oracle_idamax(x.size, _dp(x), 1)

    def dgetrf(self, A, nb: int = 64):
        _check_f64(A)
        m, n = A.shape
        piv = np.zeros(max(1, min(m, n)), dtype=np.int32)
        info = self.lib.oracle_dgetrf_nb(m, n, _dp(A), max(1, m), _ip(piv), nb)
        return piv[: min(m, n)], info

    def dgetrf_gaps(self, A):
        """dgetrf (nb = 64) that also returns, per pivot search, the relative
        gap (|first| - |second|) / |first| of the two largest candidates."""
        _check_f64(A)
        m, n = A.shape
        mn = min(m, n)
        piv = np.zeros(max(1, mn), dtype=np.int32)
        gap = np.zeros(max(1, mn), dtype=np.float64)
        info = self.lib.oracle_dgetrf_gaps(m, n, _dp(A), max(1, m), _ip(piv), _dp(gap))
        return piv[:mn], info, gap[:mn]

    def dgetrs(self, trans, LU, piv, B):
        _check_f64(LU), _check_f64(B)
        n = LU.shape[0]
        piv = np.ascontiguousarray(piv, dtype=np.int32)
        self.lib.oracle_dgetrs(trans.encode(), n, B.shape[1], _dp(LU), max(1, n),
                               _ip(piv), _dp(B), max(1, n))
        return B

    def dgesv(self, A, B):
        _check_f64(A), _check_f64(B)
        n = A.shape[0]
        piv = np.zeros(max(1, n), dtype=np.int32)
        info = self.lib.oracle_dgesv(n, B.shape[1], _dp(A), max(1, n), _ip(piv),
                                     _dp(B), max(1, n))
        return piv[:n], info

    # -- Cholesky and syrk --------------------------------------------------
    def dsyrk(self, uplo, trans, alpha, A, beta, C):
        _check_f64(A), _check_f64(C)
        n = C.shape[0]
        k = A.shape[1] if trans.upper() == "N" else A.shape[0]
        self.lib.oracle_dsyrk(uplo.encode(), trans.encode(), n, k, alpha, _dp(A),
                              max(1, A.shape[0]), beta, _dp(C), max(1, n))
        return C

    def dtrmm(self, side, uplo, transA, diag, alpha, A, B):
        _check_f64(A), _check_f64(B)
        m, n = B.shape
        self.lib.oracle_dtrmm(side.encode(), uplo.encode(), transA.encode(), diag.encode(), m, n,
                              alpha, _dp(A), max(1, A.shape[0]), _dp(B), max(1, m))
        return B

    def dsymm(self, side, uplo, alpha, A, B, beta, C):
        _check_f64(A), _check_f64(B), _check_f64(C)
        m, n = C.shape
        self.lib.oracle_dsymm(side.encode(), uplo.encode(), m, n, alpha, _dp(A),
                              max(1, A.shape[0]), _dp(B), max(1, m), beta, _dp(C), max(1, m))
        return C

    def dsyr2k(self, uplo, trans, alpha, A, B, beta, C):
        _check_f64(A), _check_f64(B), _check_f64(C)
        n = C.shape[0]
        k = A.shape[1] if trans.upper() == "N" else A.shape[0]
        self.lib.oracle_dsyr2k(uplo.encode(), trans.encode(), n, k, alpha, _dp(A),
                               max(1, A.shape[0]), _dp(B), max(1, B.shape[0]), beta, _dp(C),
                               max(1, n))
        return C

    def dtrtri(self, uplo, diag, A, nb: int = 64):
        _check_f64(A)
        n = A.shape[0]
        return self.lib.oracle_dtrtri_nb(uplo.encode(), diag.encode(), n, _dp(A), max(1, n), nb)

    def dgetri(self, A, piv):
        _check_f64(A)
        n = A.shape[0]
        piv = np.ascontiguousarray(piv, dtype=np.int32)
        return self.lib.oracle_dgetri(n, _dp(A), max(1, n), _ip(piv))

    # -- refinement, condition estimate, equilibration, expert driver -------
    def dlange(self, norm, A):
        return self.lib.oracle_dlange(norm.encode(), A.shape[0], A.shape[1], _dp(A), max(1, A.shape[0]))

    def dgecon(self, norm, LU, anorm):
        n = LU.shape[0]
        rc = ctypes.c_double(0.0)
        st = self.lib.oracle_dgecon(norm.encode(), n, _dp(LU), max(1, n), anorm, ctypes.byref(rc))
        return rc.value, st

    def dgerfs(self, trans, A, LU, piv, B, X):
        n, k = B.shape
        ferr, berr = np.zeros(max(1, k)), np.zeros(max(1, k))
        piv = np.ascontiguousarray(piv, dtype=np.int32)
        self.lib.oracle_dgerfs(trans.encode(), n, k, _dp(A), max(1, n), _dp(LU), max(1, n), _ip(piv),
                               _dp(B), max(1, n), _dp(X), max(1, n), _dp(ferr), _dp(berr))
        return ferr[:k], berr[:k]

    def dgeequ(self, A):
        m, n = A.shape
        r, c = np.zeros(max(1, m)), np.zeros(max(1, n))
        rc, cc, am = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        info = self.lib.oracle_dgeequ(m, n, _dp(A), max(1, m), _dp(r), _dp(c), ctypes.byref(rc),
                                      ctypes.byref(cc), ctypes.byref(am))
        return r[:m], c[:n], rc.value, cc.value, am.value, info

    def dlaqge(self, A, r, c, rowcnd, colcnd, amax):
        m, n = A.shape
        r = np.ascontiguousarray(r, dtype=np.float64)
        c = np.ascontiguousarray(c, dtype=np.float64)
        return self.lib.oracle_dlaqge(m, n, _dp(A), max(1, m), _dp(r), _dp(c), rowcnd, colcnd,
                                      amax).decode()

    def dgesvx(self, fact, trans, A, AF, piv, equed, r, c, B, X):
        n, k = B.shape
        eq = ctypes.create_string_buffer(equed.encode(), 2)
        rc, g = ctypes.c_double(0.0), ctypes.c_double(0.0)
        ferr, berr = np.zeros(max(1, k)), np.zeros(max(1, k))
        info = self.lib.oracle_dgesvx(fact.encode(), trans.encode(), n, k, _dp(A), max(1, n),
                                      _dp(AF), max(1, n), _ip(piv), eq, _dp(r), _dp(c), _dp(B),
                                      max(1, n), _dp(X), max(1, n), ctypes.byref(rc), _dp(ferr),
                                      _dp(berr), ctypes.byref(g))
        return info, eq.value.decode(), rc.value, ferr[:k], berr[:k], g.value

    def dpotrf(self, uplo, A, nb: int = 64):
        _check_f64(A)
        n = A.shape[0]
        return self.lib.oracle_dpotrf_nb(uplo.encode(), n, _dp(A), max(1, n), nb)

    def dpotrs(self, uplo, A, B):
        _check_f64(A), _check_f64(B)
        n = A.shape[0]
        self.lib.oracle_dpotrs(uplo.encode(), n, B.shape[1], _dp(A), max(1, n), _dp(B),
                               max(1, n))
        return B

    def dposv(self, uplo, A, B):
        _check_f64(A), _check_f64(B)
        n = A.shape[0]
        return self.lib.oracle_dposv(uplo.encode(), n, B.shape[1], _dp(A), max(1, n), _dp(B),
                                     max(1, n))

    # -- timing (CPU baseline) ---------------------------------------------
    def time_dgetrf_steps(self, n, n_blocks, n_threads, seed=1234):
        fl = ctypes.c_double(0.0)
        t = self.lib.oracle_time_dgetrf_steps(n, n_blocks, n_threads, seed,
                                              ctypes.byref(fl))
        return t, fl.value

    def time_dgetrf_step_at(self, n, block, n_threads, seed=1234):
        """(seconds, flops) of block step `block` of an n x n LU, per thread."""
        fl = ctypes.c_double(0.0)
        t = self.lib.oracle_time_dgetrf_step_at(n, block, n_threads, seed, ctypes.byref(fl))
        return t, fl.value

    def time_dgemm_rows(self, m, n, k, rows, n_threads, seed=1234):
        return self.lib.oracle_time_dgemm_rows(m, n, k, rows, n_threads, seed)


class Reference:
    """ctypes view of the reference's own Fortran-ABI shims (oracle/_ref)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        cp = ctypes.c_char_p
        L.dgemm_.argtypes = [cp, cp, _c_int_p, _c_int_p, _c_int_p, _c_double_p,
                             _c_double_p, _c_int_p, _c_double_p, _c_int_p,
                             _c_double_p, _c_double_p, _c_int_p]
        L.dtrsm_.argtypes = [cp, cp, cp, cp, _c_int_p, _c_int_p, _c_double_p,
                             _c_double_p, _c_int_p, _c_double_p, _c_int_p]
        L.dgetrf_.argtypes = [_c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_int_p,
                              _c_int_p]
        L.dgetrs_.argtypes = [cp, _c_int_p, _c_int_p, _c_double_p, _c_int_p,
                              _c_int_p, _c_double_p, _c_int_p, _c_int_p]
        L.dgesv_.argtypes = [_c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_int_p,
                             _c_double_p, _c_int_p, _c_int_p]
        L.dsyrk_.argtypes = [cp, cp, _c_int_p, _c_int_p, _c_double_p, _c_double_p, _c_int_p,
                             _c_double_p, _c_double_p, _c_int_p]
        L.dpotrf_.argtypes = [cp, _c_int_p, _c_double_p, _c_int_p, _c_int_p]
        L.dtrmm_.argtypes = [cp, cp, cp, cp, _c_int_p, _c_int_p, _c_double_p, _c_double_p,
                             _c_int_p, _c_double_p, _c_int_p]
        L.dtrtri_.argtypes = [cp, cp, _c_int_p, _c_double_p, _c_int_p, _c_int_p]
        L.dgecon_.argtypes = [cp, _c_int_p, _c_double_p, _c_int_p, _c_double_p, _c_double_p,
                              _c_double_p, _c_int_p, _c_int_p]
        L.dgerfs_.argtypes = [cp, _c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p, _c_int_p,
                              _c_int_p, _c_double_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p,
                              _c_double_p, _c_double_p, _c_int_p, _c_int_p]
        L.dgeequ_.argtypes = [_c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p, _c_double_p,
                              _c_double_p, _c_double_p, _c_double_p, _c_int_p]
        L.dlaqge_.argtypes = [_c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p, _c_double_p,
                              _c_double_p, _c_double_p, _c_double_p, ctypes.c_char_p]
        L.dgesvx_.argtypes = [cp, cp, _c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p,
                              _c_int_p, _c_int_p, ctypes.c_char_p, _c_double_p, _c_double_p,
                              _c_double_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p,
                              _c_double_p, _c_double_p, _c_double_p, _c_int_p, _c_int_p]
        L.dgetri_.argtypes = [_c_int_p, _c_double_p, _c_int_p, _c_int_p, _c_double_p, _c_int_p,
                              _c_int_p]
        L.dsymm_.argtypes = [cp, cp, _c_int_p, _c_int_p, _c_double_p, _c_double_p, _c_int_p,
                             _c_double_p, _c_int_p, _c_double_p, _c_double_p, _c_int_p]
        L.dsyr2k_.argtypes = [cp, cp, _c_int_p, _c_int_p, _c_double_p, _c_double_p, _c_int_p,
                              _c_double_p, _c_int_p, _c_double_p, _c_double_p, _c_int_p]
        L.dpotrs_.argtypes = [cp, _c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p,
                              _c_int_p, _c_int_p]
        L.dposv_.argtypes = [cp, _c_int_p, _c_int_p, _c_double_p, _c_int_p, _c_double_p,
                             _c_int_p, _c_int_p]
        L.ref_xerbla_calls.restype = ctypes.c_int
        L.ref_xerbla_info.restype = ctypes.c_int
        L.ref_xerbla_name.restype = ctypes.c_char_p

    @staticmethod
    def _i(v):
        return ctypes.byref(ctypes.c_int(int(v)))

    @staticmethod
    def _d(v):
        return ctypes.byref(ctypes.c_double(float(v)))

    def dgemm(self, transA, transB, alpha, A, B, beta, C):
        _check_f64(A), _check_f64(B), _check_f64(C)
        m, n = C.shape
        k = A.shape[1] if transA.upper() == "N" else A.shape[0]
        self.lib.dgemm_(transA.encode(), transB.encode(), self._i(m), self._i(n),
                        self._i(k), self._d(alpha), _dp(A), self._i(max(1, A.shape[0])),
                        _dp(B), self._i(max(1, B.shape[0])), self._d(beta), _dp(C),
                        self._i(max(1, m)))
        return C

    def dtrsm(self, side, uplo, transA, diag, alpha, A, B):
        _check_f64(A), _check_f64(B)
        m, n = B.shape
        self.lib.dtrsm_(side.encode(), uplo.encode(), transA.encode(), diag.encode(),
                        self._i(m), self._i(n), self._d(alpha), _dp(A),
                        self._i(max(1, A.shape[0])), _dp(B), self._i(max(1, m)))
        return B

    def dgetrf(self, A):
        _check_f64(A)
        m, n = A.shape
        piv = np.zeros(max(1, min(m, n)), dtype=np.int32)
        info = ctypes.c_int(0)
        self.lib.dgetrf_(self._i(m), self._i(n), _dp(A), self._i(max(1, m)), _ip(piv),
                         ctypes.byref(info))
        return piv[: min(m, n)], info.value

    def dgetrs(self, trans, LU, piv, B):
        n = LU.shape[0]
        piv = np.ascontiguousarray(piv, dtype=np.int32)
        info = ctypes.c_int(0)
        self.lib.dgetrs_(trans.encode(), self._i(n), self._i(B.shape[1]), _dp(LU),
                         self._i(max(1, n)), _ip(piv), _dp(B), self._i(max(1, n)),
                         ctypes.byref(info))
        return B, info.value

    def dgesv(self, A, B):
        n = A.shape[0]
        piv = np.zeros(max(1, n), dtype=np.int32)
        info = ctypes.c_int(0)
        self.lib.dgesv_(self._i(n), self._i(B.shape[1]), _dp(A), self._i(max(1, n)),
                        _ip(piv), _dp(B), self._i(max(1, n)), ctypes.byref(info))
        return piv[:n], info.value


    def dsyrk(self, uplo, trans, alpha, A, beta, C):
        n = C.shape[0]
        k = A.shape[1] if trans.upper() == "N" else A.shape[0]
        self.lib.dsyrk_(uplo.encode(), trans.encode(), self._i(n), self._i(k), self._d(alpha),
                        _dp(A), self._i(max(1, A.shape[0])), self._d(beta), _dp(C),
                        self._i(max(1, n)))
        return C

    def dtrmm(self, side, uplo, transA, diag, alpha, A, B):
        m, n = B.shape
        self.lib.dtrmm_(side.encode(), uplo.encode(), transA.encode(), diag.encode(),
                        self._i(m), self._i(n), self._d(alpha), _dp(A),
                        self._i(max(1, A.shape[0])), _dp(B), self._i(max(1, m)))
        return B

    def dsymm(self, side, uplo, alpha, A, B, beta, C):
        m, n = C.shape
        self.lib.dsymm_(side.encode(), uplo.encode(), self._i(m), self._i(n), self._d(alpha),
                        _dp(A), self._i(max(1, A.shape[0])), _dp(B), self._i(max(1, m)),
                        self._d(beta), _dp(C), self._i(max(1, m)))
        return C

    def dsyr2k(self, uplo, trans, alpha, A, B, beta, C):
        n = C.shape[0]
        k = A.shape[1] if trans.upper() == "N" else A.shape[0]
        self.lib.dsyr2k_(uplo.encode(), trans.encode(), self._i(n), self._i(k), self._d(alpha),
                         _dp(A), self._i(max(1, A.shape[0])), _dp(B), self._i(max(1, B.shape[0])),
                         self._d(beta), _dp(C), self._i(max(1, n)))
        return C

    def dgecon(self, norm, LU, anorm):
        n = LU.shape[0]
        rc, info = ctypes.c_double(0.0), ctypes.c_int(0)
        work, iwork = np.zeros(max(1, 4 * n)), np.zeros(max(1, n), dtype=np.int32)
        self.lib.dgecon_(norm.encode(), self._i(n), _dp(LU), self._i(max(1, n)), self._d(anorm),
                         ctypes.byref(rc), _dp(work), _ip(iwork), ctypes.byref(info))
        return rc.value, info.value

    def dgerfs(self, trans, A, LU, piv, B, X):
        n, k = B.shape
        ferr, berr = np.zeros(max(1, k)), np.zeros(max(1, k))
        work, iwork = np.zeros(max(1, 3 * n)), np.zeros(max(1, n), dtype=np.int32)
        piv = np.ascontiguousarray(piv, dtype=np.int32)
        info = ctypes.c_int(0)
        self.lib.dgerfs_(trans.encode(), self._i(n), self._i(k), _dp(A), self._i(max(1, n)), _dp(LU),
                         self._i(max(1, n)), _ip(piv), _dp(B), self._i(max(1, n)), _dp(X),
                         self._i(max(1, n)), _dp(ferr), _dp(berr), _dp(work), _ip(iwork),
                         ctypes.byref(info))
        return ferr[:k], berr[:k]

    def dgeequ(self, A):
        m, n = A.shape
        r, c = np.zeros(max(1, m)), np.zeros(max(1, n))
        rc, cc, am, info = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self.lib.dgeequ_(self._i(m), self._i(n), _dp(A), self._i(max(1, m)), _dp(r), _dp(c),
                         ctypes.byref(rc), ctypes.byref(cc), ctypes.byref(am), ctypes.byref(info))
        return r[:m], c[:n], rc.value, cc.value, am.value, info.value

    def dlaqge(self, A, r, c, rowcnd, colcnd, amax):
        m, n = A.shape
        r = np.ascontiguousarray(r, dtype=np.float64)
        c = np.ascontiguousarray(c, dtype=np.float64)
        eq = ctypes.create_string_buffer(b"?", 2)
        self.lib.dlaqge_(self._i(m), self._i(n), _dp(A), self._i(max(1, m)), _dp(r), _dp(c),
                         self._d(rowcnd), self._d(colcnd), self._d(amax), eq)
        return eq.value.decode()

    def dgesvx(self, fact, trans, A, AF, piv, equed, r, c, B, X):
        n, k = B.shape
        eq = ctypes.create_string_buffer(equed.encode(), 2)
        rc, info = ctypes.c_double(0.0), ctypes.c_int(0)
        ferr, berr = np.zeros(max(1, k)), np.zeros(max(1, k))
        work, iwork = np.zeros(max(1, 4 * n)), np.zeros(max(1, n), dtype=np.int32)
        self.lib.dgesvx_(fact.encode(), trans.encode(), self._i(n), self._i(k), _dp(A),
                         self._i(max(1, n)), _dp(AF), self._i(max(1, n)), _ip(piv), eq, _dp(r),
                         _dp(c), _dp(B), self._i(max(1, n)), _dp(X), self._i(max(1, n)),
                         ctypes.byref(rc), _dp(ferr), _dp(berr), _dp(work), _ip(iwork),
                         ctypes.byref(info))
        return info.value, eq.value.decode(), rc.value, ferr[:k], berr[:k], work[0]

    def dtrtri(self, uplo, diag, A):
        """The reference's dtrtri_ (flens/lapack/interface/src/trtri.cc:9-55)
        discards tri's return value: INFO is 0 for every valid call."""
        n = A.shape[0]
        info = ctypes.c_int(0)
        self.lib.dtrtri_(uplo.encode(), diag.encode(), self._i(n), _dp(A), self._i(max(1, n)),
                         ctypes.byref(info))
        return info.value

    def dgetri(self, A, piv):
        """dgetri_ with the optimal workspace (n*64); INFO is 0 for every valid
        call (flens/lapack/interface/src/getri.cc:10-53 discards tri's value)."""
        n = A.shape[0]
        piv = np.ascontiguousarray(piv, dtype=np.int32)
        work = np.zeros(max(1, n * 64))
        info = ctypes.c_int(0)
        self.lib.dgetri_(self._i(n), _dp(A), self._i(max(1, n)), _ip(piv), _dp(work),
                         self._i(work.size), ctypes.byref(info))
        return info.value

    def dpotrf(self, uplo, A):
        n = A.shape[0]
        info = ctypes.c_int(0)
        self.lib.dpotrf_(uplo.encode(), self._i(n), _dp(A), self._i(max(1, n)),
                         ctypes.byref(info))
        return info.value

    def dpotrs(self, uplo, A, B):
        n = A.shape[0]
        info = ctypes.c_int(0)
        self.lib.dpotrs_(uplo.encode(), self._i(n), self._i(B.shape[1]), _dp(A),
                         self._i(max(1, n)), _dp(B), self._i(max(1, n)), ctypes.byref(info))
        return B, info.value

    def dposv(self, uplo, A, B):
        """The reference's dposv_ (flens/lapack/interface/src/posv.cc:13-51, the call at :50)
        discards posv's return value: INFO is 0 for every valid call."""
        n = A.shape[0]
        info = ctypes.c_int(0)
        self.lib.dposv_(uplo.encode(), self._i(n), self._i(B.shape[1]), _dp(A),
                        self._i(max(1, n)), _dp(B), self._i(max(1, n)), ctypes.byref(info))
        return info.value


def reference_available() -> bool:
    return os.path.exists(REF_SO)


# -------------------------------------------------------------- inputs --
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix_uniform(seed: int, m: int, n: int) -> np.ndarray:
    """Column-major m x n matrix, entries uniform in [-1,1), from splitmix64.

    Element e (column-major position) is 2*u-1 with u = (splitmix64(seed, e) >> 11) * 2^-53.
    Pure integer arithmetic, so the same on every machine and numpy version;
    the fixtures in tests/golden store only the reference's outputs for it.
    """
    with np.errstate(over="ignore"):
        e = np.arange(m * n, dtype=np.uint64)
        z = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)) + (e + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return np.asfortranarray((2.0 * u - 1.0).reshape((n, m)).T)


def uniform(rng, m: int, n: int) -> np.ndarray:
    """uniform[-1,1] entries, column-major (rng: numpy Generator or an int seed)."""
    if isinstance(rng, (int, np.integer)):
        return splitmix_uniform(int(rng), m, n)
    return np.asfortranarray(rng.uniform(-1.0, 1.0, size=(m, n)))


def shifted_square(rng, n: int) -> np.ndarray:
    """uniform[-1,1] + (n/4) I: the well-separated-pivot input of the LU configs."""
    A = uniform(rng, n, n)
    A[np.arange(n), np.arange(n)] += n / 4.0
    return A


# -------------------------------------------------------------- metrics --
EPS64 = np.finfo(np.float64).eps


def lu_backward_error(A0: np.ndarray, LU: np.ndarray, piv: np.ndarray) -> float:
    """||P A - L U||_1 / (n ||A||_1 eps), the LAPACK dget01 style ratio."""
    m, n = A0.shape
    mn = min(m, n)
    L = np.tril(LU[:, :mn], -1) + np.eye(m, mn)
    U = np.triu(LU[:mn, :])
    PA = A0.copy()
    for i in range(mn):
        p = int(piv[i]) - 1
        if p != i:
            PA[[i, p], :] = PA[[p, i], :]
    r = np.abs(PA - L @ U).sum(axis=0).max()
    an = max(np.abs(A0).sum(axis=0).max(), np.finfo(float).tiny)
    return float(r / (max(n, 1) * an * EPS64))


def normwise_rel(X: np.ndarray, Y: np.ndarray) -> float:
    d = np.linalg.norm(X - Y)
    s = np.linalg.norm(Y)
    return float(d / s) if s > 0 else float(d)
