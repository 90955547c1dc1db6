"""C-ABI checks that need no GPU.

* libflens_gb300.so loads and exports every function include/flens_gb300.h
  declares.
* Argument checking follows the reference shims: the same parameter
  positions go to xerbla_ (flens/blas/interface/blas/gemm.cc:158-181,
  trsm.cc:136-160) and INFO=-pos for the LAPACK routines
  (flens/lapack/interface/src/getrf.cc:22-35, getrs.cc:25-40, gesv.cc:25-40).
  These checks run before any CUDA call.
* Without a GPU the compute paths fail loudly with FLENS_GB300_ERR_NO_DEVICE
  rather than falling back to the CPU.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import flens_gb300 as fg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "flens_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)))


def test_header_lists_the_entry_points():
    names = declared_functions()
    for f in ("dgemm_", "dtrsm_", "dgetrf_", "dgetrs_", "dgesv_", "flens_gb300_dgetrf"):
        assert f in names


def test_library_exports_every_declared_symbol(flib):
    missing = [n for n in declared_functions() if not hasattr(flib, n)]
    assert not missing, missing


def _i(v):
    return ctypes.byref(ctypes.c_int(v))


def _d(v):
    return ctypes.byref(ctypes.c_double(v))


NULLD = ctypes.POINTER(ctypes.c_double)()
NULLI = ctypes.POINTER(ctypes.c_int)()


def _xerbla_after(fn):
    L = fg.lib()
    before = L.flens_gb300_xerbla_calls()
    fn()
    assert L.flens_gb300_xerbla_calls() == before + 1
    return L.flens_gb300_xerbla_name().decode().strip(), L.flens_gb300_xerbla_info()


@pytest.mark.parametrize("args,pos", [
    (("X", "N", 2, 2, 2, 2, 2, 2), 1),
    (("N", "Q", 2, 2, 2, 2, 2, 2), 2),
    (("N", "N", -1, 2, 2, 2, 2, 2), 3),
    (("N", "N", 2, -1, 2, 2, 2, 2), 4),
    (("N", "N", 2, 2, -1, 2, 2, 2), 5),
    (("N", "N", 3, 2, 2, 2, 2, 3), 8),
    (("T", "N", 2, 2, 3, 2, 3, 2), 8),
    (("N", "N", 2, 2, 3, 2, 2, 2), 10),
    (("N", "N", 3, 2, 2, 3, 2, 2), 13),
])
def test_dgemm_argument_errors(capfd, args, pos):
    ta, tb, m, n, k, lda, ldb, ldc = args
    name, info = _xerbla_after(lambda: fg.lib().dgemm_(
        ta.encode(), tb.encode(), _i(m), _i(n), _i(k), _d(1.0), NULLD, _i(lda), NULLD, _i(ldb),
        _d(0.0), NULLD, _i(ldc)))
    assert name == "DGEMM" and info == pos
    assert "DGEMM" in capfd.readouterr().err


@pytest.mark.parametrize("args,pos", [
    (("X", "U", "N", "N", 2, 2, 2, 2), 1),
    (("L", "X", "N", "N", 2, 2, 2, 2), 2),
    (("L", "U", "X", "N", 2, 2, 2, 2), 3),
    (("L", "U", "N", "X", 2, 2, 2, 2), 4),
    (("L", "U", "N", "N", -1, 2, 2, 2), 5),
    (("L", "U", "N", "N", 2, -1, 2, 2), 6),
    (("L", "U", "N", "N", 3, 2, 2, 3), 9),
    (("R", "U", "N", "N", 2, 3, 2, 2), 9),
    (("L", "U", "N", "N", 3, 2, 3, 2), 11),
])
def test_dtrsm_argument_errors(args, pos):
    side, uplo, ta, diag, m, n, lda, ldb = args
    name, info = _xerbla_after(lambda: fg.lib().dtrsm_(
        side.encode(), uplo.encode(), ta.encode(), diag.encode(), _i(m), _i(n), _d(1.0), NULLD,
        _i(lda), NULLD, _i(ldb)))
    assert name == "DTRSM" and info == pos


def test_lapack_argument_errors():
    L = fg.lib()
    info = ctypes.c_int(0)
    for (m, n, lda, want) in [(-1, 2, 2, -1), (2, -1, 2, -2), (3, 2, 2, -4)]:
        name, pos = _xerbla_after(lambda: L.dgetrf_(_i(m), _i(n), NULLD, _i(lda), NULLI,
                                                    ctypes.byref(info)))
        assert info.value == want and name == "DGETRF" and pos == -want
    for (tr, n, nrhs, lda, ldb, want) in [("X", 2, 1, 2, 2, -1), ("N", -1, 1, 2, 2, -2),
                                          ("N", 2, -1, 2, 2, -3), ("N", 3, 1, 2, 3, -5),
                                          ("N", 3, 1, 3, 2, -8)]:
        name, pos = _xerbla_after(lambda: L.dgetrs_(tr.encode(), _i(n), _i(nrhs), NULLD, _i(lda),
                                                    NULLI, NULLD, _i(ldb), ctypes.byref(info)))
        assert info.value == want and name == "DGETRS" and pos == -want
    for (n, nrhs, lda, ldb, want) in [(-1, 1, 2, 2, -1), (2, -1, 2, 2, -2), (3, 1, 2, 3, -4),
                                      (3, 1, 3, 2, -7)]:
        name, pos = _xerbla_after(lambda: L.dgesv_(_i(n), _i(nrhs), NULLD, _i(lda), NULLI, NULLD,
                                                   _i(ldb), ctypes.byref(info)))
        assert info.value == want and name == "DGESV" and pos == -want


@pytest.mark.parametrize("args,pos", [
    (("X", "N", 2, 2, 2, 2), 1),
    (("L", "X", 2, 2, 2, 2), 2),
    (("L", "N", -1, 2, 2, 2), 3),
    (("L", "N", 2, -1, 2, 2), 4),
    (("L", "N", 3, 2, 2, 3), 7),
    (("U", "T", 2, 3, 2, 2), 7),
    (("L", "N", 3, 2, 3, 2), 10),
])
def test_dsyrk_argument_errors(args, pos):
    uplo, tr, n, k, lda, ldc = args
    name, info = _xerbla_after(lambda: fg.lib().dsyrk_(
        uplo.encode(), tr.encode(), _i(n), _i(k), _d(1.0), NULLD, _i(lda), _d(0.0), NULLD, _i(ldc)))
    assert name == "DSYRK" and info == pos


@pytest.mark.parametrize("fn,args,pos", [
    ("dtrmm_", ("X", "U", "N", "N", 2, 2, 2, 2), 1),
    ("dtrmm_", ("L", "X", "N", "N", 2, 2, 2, 2), 2),
    ("dtrmm_", ("L", "U", "X", "N", 2, 2, 2, 2), 3),
    ("dtrmm_", ("L", "U", "N", "X", 2, 2, 2, 2), 4),
    ("dtrmm_", ("L", "U", "N", "N", -1, 2, 2, 2), 5),
    ("dtrmm_", ("L", "U", "N", "N", 2, -1, 2, 2), 6),
    ("dtrmm_", ("R", "U", "N", "N", 2, 3, 2, 2), 9),
    ("dtrmm_", ("L", "U", "N", "N", 3, 2, 3, 2), 11),
])
def test_dtrmm_argument_errors(fn, args, pos):
    side, uplo, ta, diag, m, n, lda, ldb = args
    name, info = _xerbla_after(lambda: fg.lib().dtrmm_(
        side.encode(), uplo.encode(), ta.encode(), diag.encode(), _i(m), _i(n), _d(1.0), NULLD,
        _i(lda), NULLD, _i(ldb)))
    assert name == "DTRMM" and info == pos


@pytest.mark.parametrize("args,pos", [
    (("X", "U", 2, 2, 2, 2, 2), 1), (("L", "X", 2, 2, 2, 2, 2), 2), (("L", "U", -1, 2, 2, 2, 2), 3),
    (("L", "U", 2, -1, 2, 2, 2), 4), (("R", "U", 2, 3, 2, 2, 2), 7), (("L", "U", 3, 2, 3, 2, 3), 9),
    (("L", "U", 3, 2, 3, 3, 2), 12),
])
def test_dsymm_argument_errors(args, pos):
    side, uplo, m, n, lda, ldb, ldc = args
    name, info = _xerbla_after(lambda: fg.lib().dsymm_(
        side.encode(), uplo.encode(), _i(m), _i(n), _d(1.0), NULLD, _i(lda), NULLD, _i(ldb), _d(0.0),
        NULLD, _i(ldc)))
    assert name == "DSYMM" and info == pos


@pytest.mark.parametrize("args,pos", [
    (("X", "N", 2, 2, 2, 2, 2), 1), (("L", "X", 2, 2, 2, 2, 2), 2), (("L", "N", -1, 2, 2, 2, 2), 3),
    (("L", "N", 2, -1, 2, 2, 2), 4), (("L", "N", 3, 2, 2, 3, 3), 7), (("U", "T", 2, 3, 3, 2, 2), 9),
    (("L", "N", 3, 2, 3, 3, 2), 12),
])
def test_dsyr2k_argument_errors(args, pos):
    uplo, tr, n, k, lda, ldb, ldc = args
    name, info = _xerbla_after(lambda: fg.lib().dsyr2k_(
        uplo.encode(), tr.encode(), _i(n), _i(k), _d(1.0), NULLD, _i(lda), NULLD, _i(ldb), _d(0.0),
        NULLD, _i(ldc)))
    assert name == "DSYR2K" and info == pos


def test_cholesky_argument_errors():
    # flens/lapack/interface/src/{potrf,potrs,posv}.cc: UPLO exactly 'U' or 'L'
    L = fg.lib()
    info = ctypes.c_int(0)
    for (uplo, n, lda, want) in [("X", 2, 2, -1), ("l", 2, 2, -1), ("L", -1, 2, -2), ("U", 3, 2, -4)]:
        name, pos = _xerbla_after(lambda: L.dpotrf_(uplo.encode(), _i(n), NULLD, _i(lda),
                                                    ctypes.byref(info)))
        assert info.value == want and name == "DPOTRF" and pos == -want
    for f, nm in ((L.dpotrs_, "DPOTRS"), (L.dposv_, "DPOSV")):
        for (uplo, n, nrhs, lda, ldb, want) in [("u", 2, 1, 2, 2, -1), ("L", -1, 1, 2, 2, -2),
                                                ("L", 2, -1, 2, 2, -3), ("U", 3, 1, 2, 3, -5),
                                                ("L", 3, 1, 3, 2, -7)]:
            name, pos = _xerbla_after(lambda: f(uplo.encode(), _i(n), _i(nrhs), NULLD, _i(lda),
                                                NULLD, _i(ldb), ctypes.byref(info)))
            assert info.value == want and name == nm and pos == -want


def test_inverse_argument_errors_and_query():
    # flens/lapack/interface/src/trtri.cc:19-31, getri.cc:20-37
    L = fg.lib()
    info = ctypes.c_int(0)
    for (uplo, diag, n, lda, want) in [("X", "N", 2, 2, -1), ("u", "N", 2, 2, -1), ("U", "X", 2, 2, -2),
                                       ("U", "n", 2, 2, -2), ("L", "N", -1, 2, -3), ("L", "U", 3, 2, -5)]:
        name, pos = _xerbla_after(lambda: L.dtrtri_(uplo.encode(), diag.encode(), _i(n), NULLD,
                                                    _i(lda), ctypes.byref(info)))
        assert info.value == want and name == "DTRTRI" and pos == -want
    work = (ctypes.c_double * 1)()
    for (n, lda, lwork, want) in [(-1, 2, 2, -1), (3, 2, 3, -3), (3, 3, 2, -6)]:
        name, pos = _xerbla_after(lambda: L.dgetri_(_i(n), NULLD, _i(lda), NULLI, work, _i(lwork),
                                                    ctypes.byref(info)))
        assert info.value == want and name == "DGETRI" and pos == -want
    # workspace query: no device work, WORK(1) = N*64
    L.dgetri_(_i(100), NULLD, _i(100), NULLI, work, _i(-1), ctypes.byref(info))
    assert info.value == 0 and work[0] == 6400.0


def test_refinement_argument_errors():
    # flens/lapack/interface/src/{gerfs,gecon,geequ,gesvx}.cc
    L = fg.lib()
    info = ctypes.c_int(0)
    d = ctypes.c_double(1.0)
    for (tr, n, k, lda, ldaf, ldb, ldx, want) in [
            ("X", 2, 1, 2, 2, 2, 2, -1), ("N", -1, 1, 2, 2, 2, 2, -2), ("N", 2, -1, 2, 2, 2, 2, -3),
            ("N", 3, 1, 2, 3, 3, 3, -5), ("T", 3, 1, 3, 2, 3, 3, -7), ("N", 3, 1, 3, 3, 2, 3, -10),
            ("C", 3, 1, 3, 3, 3, 2, -12)]:
        name, pos = _xerbla_after(lambda: L.dgerfs_(
            tr.encode(), _i(n), _i(k), NULLD, _i(lda), NULLD, _i(ldaf), NULLI, NULLD, _i(ldb), NULLD,
            _i(ldx), NULLD, NULLD, NULLD, NULLI, ctypes.byref(info)))
        assert info.value == want and name == "DGERFS" and pos == -want
    for (nm, n, lda, an, want) in [("X", 2, 2, 1.0, -1), ("1", -1, 2, 1.0, -2), ("O", 3, 2, 1.0, -4),
                                   ("I", 2, 2, -1.0, -5)]:
        name, pos = _xerbla_after(lambda: L.dgecon_(nm.encode(), _i(n), NULLD, _i(lda), _d(an),
                                                    ctypes.byref(d), NULLD, NULLI, ctypes.byref(info)))
        assert info.value == want and name == "DGECON" and pos == -want
    for (m, n, lda, want) in [(-1, 2, 2, -1), (2, -1, 2, -2), (3, 2, 2, -4)]:
        name, pos = _xerbla_after(lambda: L.dgeequ_(_i(m), _i(n), NULLD, _i(lda), NULLD, NULLD,
                                                    ctypes.byref(d), ctypes.byref(d), ctypes.byref(d),
                                                    ctypes.byref(info)))
        assert info.value == want and name == "DGEEQU" and pos == -want
    eq = ctypes.create_string_buffer(b"N", 2)
    for (fact, tr, n, k, lda, ldaf, ldb, ldx, want) in [
            ("X", "N", 2, 1, 2, 2, 2, 2, -1), ("N", "X", 2, 1, 2, 2, 2, 2, -2),
            ("N", "N", -1, 1, 2, 2, 2, 2, -3), ("N", "N", 2, -1, 2, 2, 2, 2, -4),
            ("N", "N", 3, 1, 2, 3, 3, 3, -6), ("E", "N", 3, 1, 3, 2, 3, 3, -8),
            ("N", "T", 3, 1, 3, 3, 2, 3, -14), ("N", "N", 3, 1, 3, 3, 3, 2, -16)]:
        name, pos = _xerbla_after(lambda: L.dgesvx_(
            fact.encode(), tr.encode(), _i(n), _i(k), NULLD, _i(lda), NULLD, _i(ldaf), NULLI, eq,
            NULLD, NULLD, NULLD, _i(ldb), NULLD, _i(ldx), ctypes.byref(d), NULLD, NULLD, NULLD,
            NULLI, ctypes.byref(info)))
        assert info.value == want and name == "DGESVX" and pos == -want
    # FACT = 'F' with an invalid EQUED
    bad = ctypes.create_string_buffer(b"Q", 2)
    name, pos = _xerbla_after(lambda: L.dgesvx_(
        b"F", b"N", _i(2), _i(1), NULLD, _i(2), NULLD, _i(2), NULLI, bad, NULLD, NULLD, NULLD, _i(2),
        NULLD, _i(2), ctypes.byref(d), NULLD, NULLD, NULLD, NULLI, ctypes.byref(info)))
    assert info.value == -10 and name == "DGESVX"


def test_quick_returns_touch_nothing():
    # m==0 / n==0 return before any device work (gemm.tcc:54-56, trf.tcc:81-83)
    L = fg.lib()
    info = ctypes.c_int(7)
    L.dgetrf_(_i(0), _i(5), NULLD, _i(1), NULLI, ctypes.byref(info))
    assert info.value == 0
    L.dgemm_(b"N", b"N", _i(0), _i(3), _i(2), _d(1.0), NULLD, _i(1), NULLD, _i(2), _d(0.0),
             NULLD, _i(1))


def test_device_api_argument_errors_cholesky(flib):
    assert flib.flens_gb300_dpotrf(b"X", 1, None, 1, None, None) == -1
    assert flib.flens_gb300_dpotrf(b"L", 3, None, 2, None, None) == -4
    assert flib.flens_gb300_dpotrs(b"U", 2, -1, None, 2, None, 2, None) == -3
    assert flib.flens_gb300_dposv(b"L", 3, 1, None, 3, None, 2, None, None) == -7
    assert flib.flens_gb300_dsyrk(b"L", b"Q", 1, 1, 1.0, None, 1, 0.0, None, 1, None) == -2
    assert flib.flens_gb300_dsyrk(b"U", b"T", 2, 3, 1.0, None, 2, 0.0, None, 2, None) == -7


def test_device_api_argument_errors(flib):
    assert flib.flens_gb300_dgemm(b"X", b"N", 1, 1, 1, 1.0, None, 1, None, 1, 0.0, None, 1, None) == -1
    assert flib.flens_gb300_dgetrf(-1, 1, None, 1, None, None, None) == -1
    assert flib.flens_gb300_dgetrf(3, 1, None, 2, None, None, None) == -4
    assert flib.flens_gb300_dgetrs(b"N", 3, 1, None, 3, None, None, 2, None) == -8
    assert flib.flens_gb300_dgetrf_split(-1, 4, None, 4, None, None, 0, None) == -1
    assert flib.flens_gb300_dgetrf_split(4, -1, None, 4, None, None, 0, None) == -2
    assert flib.flens_gb300_dgetrf_split(4, 4, None, 3, None, None, 0, None) == -4
    assert flib.flens_gb300_dgetrf_split(4, 4, None, 4, None, None, 100, None) == -7
    assert flib.flens_gb300_dgetrf_split(4, 4, None, 4, None, None, -64, None) == -7


@pytest.mark.parametrize("prec,want", [(-1, -1), (4, -1), (7, -1)])
def test_sgemm_tc_precision_codes(flib, prec, want):
    # 0-3, 5 and 6 (two- and three-term e4m3) are product precisions; 4 names
    # the split LU of the mixed solve and is rejected here, before any CUDA call
    f = flib.flens_gb300_sgemm_tc
    f.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_char] + [ctypes.c_int] * 3 + [
        ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
        ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    assert f(prec, b"N", b"N", 4, 4, 4, 1.0, None, 4, None, 4, 0.0, None, 4, None) == want
    assert f(5, b"X", b"N", 4, 4, 4, 1.0, None, 4, None, 4, 0.0, None, 4, None) == -2


def test_dgesv_mixed_precision_codes(flib):
    f = flib.flens_gb300_dgesv_mixed
    f.argtypes = [ctypes.c_int] * 2 + [ctypes.c_void_p, ctypes.c_int] * 3 + [ctypes.c_int] * 3 + [
        ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert f(4, 1, None, 4, None, 4, None, 4, 7, 2, 0, 0.0, None, None, None, None) == -9
    assert f(4, 1, None, 4, None, 4, None, 4, -1, 2, 0, 0.0, None, None, None, None) == -9
    assert f(4, 1, None, 4, None, 4, None, 4, 5, 3, 0, 0.0, None, None, None, None) == -10


def test_sgetrf_tc_argument_errors(flib):
    f = flib.flens_gb300_sgetrf_tc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    assert f(4, 4, 4, None, 4, None, None, None) == -1
    assert f(-2, 4, 4, None, 4, None, None, None) == -1
    assert f(7, 4, 4, None, 4, None, None, None) == -1
    assert f(6, -1, 4, None, 4, None, None, None) == -2
    assert f(6, 4, -1, None, 4, None, None, None) == -3
    assert f(-1, 4, 4, None, 3, None, None, None) == -5


def _trmv_hook(flib):
    f = flib.flens_gb300_test_trmv_zeros
    f.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 7
    return f


def test_trmv_zeros_hook_arguments_and_scratch_sizes(flib):
    f = _trmv_hook(flib)
    assert f(b"X", 4, None, 4, None, None, None, None, None, None, None) == -1
    assert f(b"L", -1, None, 4, None, None, None, None, None, None, None) == -2
    assert f(b"U", 4, None, 3, None, None, None, None, None, None, None) == -4
    # the size query needs no device: one counter per 16-row block and, per
    # row, one partial sum for each chunk of the longest row (chunks of at
    # least 256 columns)
    pe, ce = ctypes.c_size_t(0), ctypes.c_size_t(0)
    for n in (1, 16, 17, 256, 257, 2048):
        assert f(b"l", n, None, n, None, None, None, None, ctypes.byref(pe), ctypes.byref(ce), None) == 0
        assert ce.value == -(-n // 16)
        assert n <= pe.value <= n * -(-n // 256)
    assert f(b"U", 0, None, 1, None, None, None, None, ctypes.byref(pe), ctypes.byref(ce), None) == 0
    assert pe.value == 0 and ce.value == 0


def test_no_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    A = np.asfortranarray(np.eye(3))
    piv, info = fg.dgetrf(A)
    assert info == fg.ERR_NO_DEVICE, (info, fg.last_error())
    assert fg.last_error() != ""


def test_batched_queries_reject_missing_plans_and_buckets(flib):
    # the plan queries answer -1 instead of reading through a null plan or past
    # the last size bucket (no CUDA call is made)
    vp = ctypes.c_void_p
    for fn in (flib.flens_gb300_batched_team, flib.flens_gb300_batched_panel):
        fn.argtypes = [vp, ctypes.c_int]
        fn.restype = ctypes.c_int
        assert fn(None, 0) == -1
        assert fn(None, -1) == -1


def test_batched_plan_argument_errors(flib):
    # argument checks before any device work: negative count, bad precision,
    # no output pointer, an illegal size in the metadata
    vp = ctypes.c_void_p
    f = flib.flens_gb300_dgesv_batched_plan
    f.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, vp, vp, ctypes.c_int,
                  vp, ctypes.POINTER(ctypes.c_void_p)]
    f.restype = ctypes.c_int
    plan = ctypes.c_void_p()
    n = np.array([4, -1], dtype=np.int32)
    k = np.array([1, 1], dtype=np.int32)
    ld = np.array([4, 4], dtype=np.int32)
    assert f(-1, None, None, None, None, None, None, None, None, 0, None, None, 0, None,
             ctypes.byref(plan)) == -1
    assert f(0, None, None, None, None, None, None, None, None, 3, None, None, 0, None,
             ctypes.byref(plan)) == -10
    assert f(0, None, None, None, None, None, None, None, None, -1, None, None, 0, None,
             ctypes.byref(plan)) == -10
    assert f(0, None, None, None, None, None, None, None, None, 0, None, None, 0, None, None) == -15
    assert f(2, n.ctypes.data, k.ctypes.data, None, ld.ctypes.data, None, None, ld.ctypes.data,
             None, 0, None, None, 0, None, ctypes.byref(plan)) == -2
    assert "illegal size" in fg.last_error()


def test_blas_failure_goes_to_the_hook_without_gpu(capfd):
    # BLAS routines have no INFO: an internal failure (here: no device) goes to
    # the caller's hook instead of stderr, and the thread's BLAS status keeps it
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = fg.lib()
    HOOK = ctypes.CFUNCTYPE(None, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p)
    seen = []
    hook = HOOK(lambda r, st, msg: seen.append((r.decode(), st, msg.decode())))
    L.flens_gb300_set_blas_error_hook.argtypes = [HOOK]
    L.flens_gb300_set_blas_error_hook.restype = None
    L.flens_gb300_blas_status.restype = ctypes.c_int
    L.flens_gb300_set_blas_error_hook(hook)
    try:
        A, B, C = (np.asfortranarray(np.ones((3, 3))) for _ in range(3))
        fg.dgemm("N", "N", 1.0, A, B, 0.0, C)
        assert L.flens_gb300_blas_status() == fg.ERR_NO_DEVICE
        assert seen and seen[-1][0] == "dgemm_" and seen[-1][1] == fg.ERR_NO_DEVICE
        assert "dgemm_ failed" not in capfd.readouterr().err
    finally:
        L.flens_gb300_set_blas_error_hook(HOOK())
    fg.dgemm("N", "N", 1.0, A, B, 0.0, C)
    assert "dgemm_ failed (-1003)" in capfd.readouterr().err


def test_allocation_diagnostics_without_gpu():
    L = fg.lib()
    L.flens_gb300_device_alloc_count.restype = ctypes.c_longlong
    L.flens_gb300_test_fail_device_allocs.argtypes = [ctypes.c_int]
    before = L.flens_gb300_device_alloc_count()
    L.flens_gb300_test_fail_device_allocs(0)
    assert L.flens_gb300_device_alloc_count() == before >= 0
