"""Precision form: low-precision LU on the tensor cores + FP64 refinement
(flens_gb300_dgesv_mixed) must reach FP64-level accuracy.

Systems follow the mixed-solve configuration: A = U diag(s) V^T, U and V the Q
factors of Householder QR of seeded Gaussian matrices, s geometric from 1 to
1/kappa, b = A x_true.  Bars (written in the asserts): the reported and the
independently recomputed normwise backward error
||b - Ax||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= 10 n eps64, and the
forward error against x_true <= kappa * 10 n eps64, kappa times the
backward-error bar: the solver stops once its backward error is below
n eps64, so the forward error can reach kappa times that (a solve that
happens to stop earlier lands lower).
"""
import ctypes

import numpy as np
import pytest

import flens_gb300 as fg

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
PREC = {"tf32": 0, "bf16": 1, "fp8": 2, "fp32": 3, "split": 4, "fp8x2": 5, "fp8x3": 6}
SOLVER = {"classical": 0, "gmres": 1, "auto": 2}


def make_system(cuda, n, kappa, nrhs, seed):
    import torch
    g = torch.Generator(device=cuda)
    g.manual_seed(seed)
    U, _ = torch.linalg.qr(torch.randn((n, n), generator=g, dtype=torch.float64, device=cuda))
    V, _ = torch.linalg.qr(torch.randn((n, n), generator=g, dtype=torch.float64, device=cuda))
    s = kappa ** (-torch.arange(n, dtype=torch.float64, device=cuda) / (n - 1))
    A = fg.to_colmajor((U * s) @ V.t())
    x = torch.rand((n, nrhs), generator=g, dtype=torch.float64, device=cuda).mul_(2).sub_(1)
    b = fg.to_colmajor(A @ x)
    return A, b, x


def dgesv_mixed(A, b, prec, solver, max_iter=30, tol=0.0):
    import torch
    n, nrhs = b.shape
    X = fg.colmajor_empty(n, nrhs, device=A.device)
    f = fg.lib().flens_gb300_dgesv_mixed
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    f.restype = ctypes.c_int
    it, be, inf = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    ld = lambda t: max(t.stride(1), t.shape[0], 1)     # one-column tensors report stride 1
    st = f(n, nrhs, A.data_ptr(), ld(A), b.data_ptr(), ld(b), X.data_ptr(), ld(X),
           PREC[prec], SOLVER[solver], max_iter, tol, ctypes.byref(it), ctypes.byref(be),
           ctypes.byref(inf), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, X, it.value, be.value, inf.value


def backward_error(A, X, b):
    r = b - A @ X
    anorm = A.abs().sum(1).max()
    return (r.abs().amax(0) / (anorm * X.abs().amax(0) + b.abs().amax(0))).max().item()


@pytest.mark.parametrize("prec", ["fp32", "tf32", "bf16", "fp8", "fp8x2", "fp8x3"])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_mixed_well_conditioned(cuda, prec, nrhs):
    n, kappa = 512, 1e2
    A, b, x = make_system(cuda, n, kappa, nrhs, 11)
    st, X, it, be, inf = dgesv_mixed(A, b, prec, "auto")
    assert st == 0 and inf == 0, (st, fg.last_error())
    assert be <= 10 * n * EPS
    assert backward_error(A, X, b) <= 10 * n * EPS
    fwd = ((X - x).abs().max() / x.abs().max()).item()
    assert fwd <= kappa * 10 * n * EPS, fwd


@pytest.mark.parametrize("solver", ["classical", "gmres", "auto"])
def test_mixed_kappa_1e6_fp32_factors(cuda, solver):
    # FP32-accurate (3xTF32) factors: kappa*u32 ~ 0.06, classical refinement converges
    n, kappa = 1024, 1e6
    A, b, x = make_system(cuda, n, kappa, 2, 12)
    st, X, it, be, inf = dgesv_mixed(A, b, "fp32", solver, max_iter=40)
    assert st == 0, (st, fg.last_error(), it, be)
    assert backward_error(A, X, b) <= 10 * n * EPS
    fwd = ((X - x).abs().max() / x.abs().max()).item()
    assert fwd <= kappa * 10 * n * EPS, fwd


def test_mixed_gmres_kappa_1e10(cuda):
    # kappa*u32 ~ 600: classical refinement diverges, GMRES-IR converges.  On
    # this matrix family (geometric singular values) GMRES needs about as many
    # iterations as there are singular values below 1/(u32*growth), so the
    # test keeps n within one restart cycle.
    n, kappa = 256, 1e10
    A, b, x = make_system(cuda, n, kappa, 1, 13)
    st, X, it, be, inf = dgesv_mixed(A, b, "fp32", "gmres", max_iter=10)
    assert st == 0, (st, fg.last_error(), it, be)
    assert backward_error(A, X, b) <= 10 * n * EPS
    fwd = ((X - x).abs().max() / x.abs().max()).item()
    assert fwd <= kappa * 10 * n * EPS, fwd


def test_mixed_auto_switches_to_gmres(cuda):
    # bf16 factors at kappa=1e2 on n=512: auto finishes (classical or GMRES-IR)
    n = 512
    A, b, x = make_system(cuda, n, 1e3, 1, 16)
    st, X, it, be, inf = dgesv_mixed(A, b, "bf16", "auto", max_iter=40)
    assert st == 0, (st, fg.last_error(), it, be)
    assert backward_error(A, X, b) <= 10 * n * EPS


def test_mixed_classical_reports_non_convergence(cuda):
    # bf16 factors of a kappa=1e10 matrix: classical refinement cannot converge
    # and must say so instead of returning a wrong "success"
    n = 512
    A, b, x = make_system(cuda, n, 1e10, 1, 14)
    st, X, it, be, inf = dgesv_mixed(A, b, "bf16", "classical", max_iter=10)
    assert st == fg.ERR_NOT_CONVERGED
    assert be > 10 * n * EPS


def test_mixed_singular_info(cuda):
    import torch
    n = 256
    A, b, x = make_system(cuda, n, 10.0, 1, 15)
    A[:, 7] = 0.0
    st, X, it, be, inf = dgesv_mixed(A, b, "bf16", "auto")
    assert st == 0 and inf == 8


def test_mixed_argument_errors(cuda):
    f = fg.lib().flens_gb300_dgesv_mixed
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p]
    assert f(-1, 1, None, 1, None, 1, None, 1, 0, 0, 5, 0.0, None, None, None, None) == -1
    assert f(4, 1, None, 3, None, 4, None, 4, 0, 0, 5, 0.0, None, None, None, None) == -4
    assert f(4, 1, None, 4, None, 4, None, 4, 7, 0, 5, 0.0, None, None, None, None) == -9


@pytest.mark.parametrize("n", [256, 300, 64, 50])
@pytest.mark.parametrize("prec", ["fp32", "split"])
def test_mixed_gmres_preconditioner_quality(cuda, n, prec):
    # GMRES-IR with well-conditioned A: with the exact preconditioner
    # (LU)^-1 A = I + O(u_f), GMRES needs a handful of iterations; a wrong
    # block (inverse, neighbour product, partial last block) would leave it
    # near n iterations.  n = 300 and 50 end in a partial 64-row block.
    A, b, x = make_system(cuda, n, 1e2, 1, 17)
    st, X, it, be, inf = dgesv_mixed(A, b, prec, "gmres", max_iter=5)
    assert st == 0, (st, fg.last_error(), it, be)
    assert it <= (12 if prec == "fp32" else 4), it
    assert backward_error(A, X, b) <= 10 * n * EPS


def test_mixed_gmres_ill_conditioned_partial_block(cuda):
    # n = 300 ends in a partial 64-row block.  kappa = 1e8 leaves about 30
    # singular values below 1/(u32*growth), within one restart cycle (at
    # kappa = 1e10 it is about 80 of 300, and restarted GMRES(100) stagnates)
    n = 300
    A, b, x = make_system(cuda, n, 1e8, 1, 13)
    st, X, it, be, inf = dgesv_mixed(A, b, "fp32", "gmres", max_iter=10)
    assert st == 0, (st, fg.last_error(), it, be)
    assert backward_error(A, X, b) <= 10 * n * EPS


def _emulated_lu_error(A64, prec, nb=64):
    """||PA - LU||_F / ||A||_F of a torch emulation of the same factorisation
    (CPU, FP64 arithmetic on FP32 storage): panels in FP64, U12 by an FP64
    triangular solve, trailing updates from the operands rounded as the
    tensor-core kind rounds them (e4m3 terms of the per-row / per-column
    scaled entries)."""
    import torch
    pairs = {"fp8x2": [(0, 0), (0, 1), (1, 0)],
             "fp8x3": [(0, 0), (0, 1), (1, 0), (0, 2), (2, 0), (1, 1)]}[prec]
    nt = 2 if prec == "fp8x2" else 3

    def terms(x):
        amax = x.abs().amax(dim=1, keepdim=True)
        s = torch.where(amax > 0, amax / 448.0, torch.ones_like(amax))
        r, out = x * (1.0 / s), []
        for _ in range(nt):
            t = r.to(torch.float8_e4m3fn).to(torch.float32)
            out.append(t.double())
            r = r - t
        return s.double(), out

    A = A64.to(torch.float32).clone()
    n = A.shape[0]
    perm = torch.arange(n)
    for j in range(0, n, nb):
        jb = min(nb, n - j)
        P = A[j:, j:j + jb].double()
        for c in range(jb):
            p = int(torch.argmax(P[c:, c].abs())) + c
            if p != c:
                P[[c, p]] = P[[p, c]]
                for sl in (slice(0, j), slice(j + jb, n)):
                    A[[j + c, j + p], sl] = A[[j + p, j + c], sl]
                perm[[j + c, j + p]] = perm[[j + p, j + c]]
            P[c + 1:, c] /= P[c, c]
            P[c + 1:, c + 1:] -= torch.outer(P[c + 1:, c], P[c, c + 1:])
        A[j:, j:j + jb] = P.to(torch.float32)
        if j + jb < n:
            L11 = torch.tril(A[j:j + jb, j:j + jb].double(), -1) + torch.eye(jb, dtype=torch.float64)
            A[j:j + jb, j + jb:] = torch.linalg.solve_triangular(
                L11, A[j:j + jb, j + jb:].double(), upper=False, unitriangular=True).to(torch.float32)
            sa, ta = terms(A[j + jb:, j:j + jb].contiguous())
            sb, tb = terms(A[j:j + jb, j + jb:].t().contiguous())
            upd = sa * sum(ta[i] @ tb[k].t() for i, k in pairs) * sb.t()
            A[j + jb:, j + jb:] = (A[j + jb:, j + jb:].double() - upd).to(torch.float32)
    L = torch.tril(A.double(), -1) + torch.eye(n, dtype=torch.float64)
    return float((A64[perm] - L @ torch.triu(A.double())).norm() / A64.norm())


def test_sgetrf_tc_factor_error_per_precision(cuda):
    """flens_gb300_sgetrf_tc on the mixed-solve matrix family (n = 512,
    kappa = 1e2): ||PA - LU||_F / ||A||_F per trailing-update precision.  The
    split e4m3 forms must match a torch emulation of the same factorisation
    to 25% (the GPU's panels and U12 solve are FP32, the emulation's FP64:
    the e4m3 product errors dominate both), and the
    precisions must order as their unit roundoffs do: FP32 (CUDA cores and
    3xTF32) << three-term e4m3 (~2^-12) < TF32 (2^-11) < two-term e4m3 and
    BF16 (~2^-8) < one-term e4m3 (2^-4)."""
    import torch
    n = 512
    A, _, _ = make_system(cuda, n, 1e2, 1, 21)
    f = fg.lib().flens_gb300_sgetrf_tc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    err = {}
    for name, prec in (("fp32", -1), ("3xtf32", 3), ("tf32", 0), ("bf16", 1), ("fp8", 2),
                       ("fp8x2", 5), ("fp8x3", 6)):
        F = A.to(torch.float32).t().contiguous().t()
        ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
        info = torch.zeros(1, dtype=torch.int32, device=cuda)
        st = f(prec, n, n, F.data_ptr(), n, ipiv.data_ptr(), info.data_ptr(),
               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        assert st == 0 and int(info.item()) == 0, (name, st, fg.last_error())
        perm = list(range(n))
        for i, p in enumerate(ipiv.cpu().numpy()):
            perm[i], perm[p - 1] = perm[p - 1], perm[i]
        Fd = F.double()
        L = torch.tril(Fd, -1) + torch.eye(n, dtype=torch.float64, device=cuda)
        err[name] = float((A[perm] - L @ torch.triu(Fd)).norm() / A.norm())
    A64 = A.cpu()
    for name in ("fp8x2", "fp8x3"):
        ref = _emulated_lu_error(A64, name)
        assert abs(err[name] - ref) <= 0.25 * ref, (name, err[name], ref)
    assert err["fp32"] < 1e-5 and err["3xtf32"] < 1e-5, err
    assert err["3xtf32"] < err["fp8x3"] < err["tf32"] < err["fp8x2"] < err["fp8"], err
    assert err["bf16"] < err["fp8"] and err["fp8x2"] < err["bf16"], err


def test_mixed_fp8x3_converges_where_fp8_cannot(cuda):
    """n = 4096, kappa = 1e2: one-term e4m3 factors are no preconditioner
    (||I - (LU)^-1 PA|| >> 1 at this size), three-term e4m3 factors reach
    10 n eps in a few steps."""
    n = 4096
    A, b, x = make_system(cuda, n, 1e2, 1, 22)
    st, X, it, be, inf = dgesv_mixed(A, b, "fp8x3", "auto")
    assert st == 0 and inf == 0, (st, fg.last_error(), it, be)
    assert it <= 10, it
    assert backward_error(A, X, b) <= 10 * n * EPS
    st1, _, it1, be1, _ = dgesv_mixed(A, b, "fp8", "auto", max_iter=4)
    assert st1 == fg.ERR_NOT_CONVERGED and be1 > 10 * n * EPS


@pytest.mark.parametrize("m,n", [(700, 300), (300, 700), (257, 257), (1000, 1000), (64, 64), (65, 130)])
@pytest.mark.parametrize("prec", [-1, 3, 1])
def test_sgetrf_tc_shapes(cuda, m, n, prec):
    """flens_gb300_sgetrf_tc on rectangular and ragged shapes (outer blocks
    of 256 columns cut short by min(m, n) or by n, panels narrower than 64):
    P A = L U with a backward error at the precision's level, unit lower L
    below the diagonal of the first min(m, n) columns, pivots in range."""
    import torch
    g = torch.Generator(device=cuda)
    g.manual_seed(m * 7 + n)
    A = (torch.rand((m, n), generator=g, dtype=torch.float64, device=cuda) * 2 - 1)
    ld = m + 3                                   # a leading dimension beyond m
    buf = torch.zeros((n, ld), dtype=torch.float32, device=cuda)
    F = buf.t()[:m, :]                           # m x n view, column stride ld
    F.copy_(A.to(torch.float32))
    mn = min(m, n)
    ipiv = torch.zeros(mn, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    f = fg.lib().flens_gb300_sgetrf_tc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    st = f(prec, m, n, buf.data_ptr(), ld, ipiv.data_ptr(), info.data_ptr(),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == 0 and int(info.item()) == 0, (st, fg.last_error())
    pv = ipiv.cpu().numpy()
    assert (pv >= np.arange(1, mn + 1)).all() and (pv <= m).all()
    perm = list(range(m))
    for i, p in enumerate(pv):
        perm[i], perm[p - 1] = perm[p - 1], perm[i]
    Fd = F.double()
    L = torch.tril(Fd, -1)[:, :mn] + torch.eye(m, mn, dtype=torch.float64, device=cuda)
    U = torch.triu(Fd)[:mn, :]
    err = ((A[perm] - L @ U).norm() / A.norm()).item()
    bound = {-1: 1e-5, 3: 1e-5, 1: 0.25}[prec]     # BF16: gross errors only
    assert err <= bound, (m, n, prec, err)
    # the padding rows beyond m are untouched
    assert (buf.t()[m:, :] == 0).all()


@pytest.mark.parametrize("prec,n", [("bf16", 2048), ("fp8x2", 2048), ("bf16", 2100)])
def test_mixed_explicit_inverse_preconditioner(cuda, prec, n):
    """BF16 and FP8 factors at n >= 2048 take GMRES with the explicit-inverse
    preconditioner (L^-1, U^-1 formed once by 3xTF32 block recursion, applied
    as FP64 products); the solve must reach 10 n eps as with the chained
    substitution (17 and 22 steps at n = 2048, kappa = 1e2).  n = 2100 leaves
    a 52-row last diagonal block, halves of the recursion that are not
    multiples of 64 and a 4-row last row block in the chunked products."""
    A, b, x = make_system(cuda, n, 1e2, 1, 23)
    st, X, it, be, inf = dgesv_mixed(A, b, prec, "auto")
    assert st == 0 and inf == 0, (st, fg.last_error(), it, be)
    assert it <= 60, it
    assert backward_error(A, X, b) <= 10 * n * EPS
    fwd = ((X - x).abs().max() / x.abs().max()).item()
    assert fwd <= 1e2 * 10 * n * EPS, fwd


@pytest.mark.parametrize("uplo", ["L", "U", "G"])
@pytest.mark.parametrize("n", [1, 17, 300, 2048, 5000])
def test_chunked_gemv_of_the_mixed_solve(cuda, uplo, n):
    """The preconditioner's product y = T x over one triangle T (the other
    holding zeros; uplo L and U) and the Arnoldi product over all of A
    (uplo G): equal to the FP64 product to rounding, bitwise the same on a
    repeated call (the chunk sums of a row block are added in chunk order
    whatever the CTAs' timing), and the row blocks' counters back at zero
    after each call.  For a triangle the kernel reads the triangle and the
    zeros of its 16 x 16 diagonal blocks, nothing else: the rest of the
    other triangle is NaN here."""
    import torch
    g = torch.Generator(device=cuda).manual_seed(n)
    T = torch.rand((n, n), generator=g, dtype=torch.float64, device=cuda) * 2 - 1
    if uplo != "G":
        T = torch.tril(T) if uplo == "L" else torch.triu(T)
    i = torch.arange(n, device=cuda).view(-1, 1) // 16
    j = torch.arange(n, device=cuda).view(1, -1) // 16
    read = (j <= i) if uplo == "L" else (j >= i) if uplo == "U" else (i >= 0) & (j >= 0)
    Tp = fg.to_colmajor(torch.where(read, T, torch.full_like(T, float("nan"))))
    x = torch.rand(n, generator=g, dtype=torch.float64, device=cuda) * 2 - 1
    f = fg.lib().flens_gb300_test_trmv_zeros
    f.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 7
    pe, ce = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert f(uplo.encode(), n, None, n, None, None, None, None, ctypes.byref(pe), ctypes.byref(ce), None) == 0
    part = torch.zeros(max(pe.value, 1), dtype=torch.float64, device=cuda)
    cnt = torch.zeros(max(ce.value, 1), dtype=torch.int32, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ys = []
    for _ in range(2):
        y = torch.full((n,), float("nan"), dtype=torch.float64, device=cuda)
        assert f(uplo.encode(), n, Tp.data_ptr(), Tp.stride(1), x.data_ptr(), y.data_ptr(),
                 part.data_ptr(), cnt.data_ptr(), None, None, stream) == 0
        torch.cuda.synchronize()
        assert int(cnt.abs().sum()) == 0
        ys.append(y.cpu().numpy())
    want = T.cpu().numpy() @ x.cpu().numpy()
    scale = np.abs(T.cpu().numpy()) @ np.abs(x.cpu().numpy())
    assert np.all(np.abs(ys[0] - want) <= 4 * n * EPS * scale + 1e-300)
    np.testing.assert_array_equal(ys[0], ys[1])
