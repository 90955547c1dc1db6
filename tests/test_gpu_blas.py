"""GPU parity for dgemm / dtrsm through the C ABI.

Bars (written in each assert): GEMM normwise relative error <= 1e-13 against
the reference's own result (the project's gemm parity bar); TRSM <= 1e-12 on
well-conditioned triangles.  Semantics that are bitwise in the reference
(alpha==0 scaling, beta multiply) are checked bitwise.
"""
import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu

GEMM_TOL = 1e-13
TRSM_TOL = 1e-12


def rel(x, y):
    if y.size == 0:
        return 0.0
    return oracle.normwise_rel(x, y)


def test_gemm_fixtures_host_api(cuda, golden):
    for i, (name, (m, n, k, ta, tb, a, b)) in enumerate(G.gemm_case_list()):
        A, B, C = G.gemm_inputs(i, m, n, k, ta, tb)
        out = fg.dgemm(ta, tb, a, A, B, b, C.copy(order="F"))
        ref = golden[name]
        if a == 0.0:
            assert np.array_equal(out, ref), name          # pure beta scaling: exact
        else:
            assert rel(out, ref) <= GEMM_TOL, (name, rel(out, ref))


def test_gemm_fixtures_device_api(cuda, golden):
    import torch
    for i, (name, (m, n, k, ta, tb, a, b)) in enumerate(G.gemm_case_list()):
        if min(m, n, k) == 0:
            continue
        A, B, C = G.gemm_inputs(i, m, n, k, ta, tb)
        dA, dB, dC = (fg.to_colmajor(torch.from_numpy(x).to(cuda)) for x in (A, B, C))
        fg.dgemm_dev(ta, tb, a, dA, dB, b, dC)
        torch.cuda.synchronize()
        assert rel(dC.cpu().numpy(), golden[name]) <= GEMM_TOL, name


def test_gemm_alpha_zero_does_not_read_A_B(cuda):
    # cxxblas/level3/gemm.tcc:66-69: scale by beta, then return when alpha==0
    A = np.asfortranarray(np.full((5, 4), np.nan))
    B = np.asfortranarray(np.full((4, 6), np.nan))
    C = oracle.uniform(3, 5, 6)
    out = fg.dgemm("N", "N", 0.0, A, B, 1.25, C.copy(order="F"))
    assert np.array_equal(out, 1.25 * C)


def test_gemm_beta_zero_multiplies(cuda, port):
    # gescal multiplies by beta, so a NaN in C survives beta == 0 (as in the reference)
    A, B = oracle.uniform(4, 6, 5), oracle.uniform(5, 5, 7)
    C = oracle.uniform(6, 6, 7)
    C[2, 3] = np.nan
    out = fg.dgemm("N", "N", 1.0, A, B, 0.0, C.copy(order="F"))
    ref = port.dgemm("N", "N", 1.0, A, B, 0.0, C.copy(order="F"))
    assert np.isnan(out[2, 3]) and np.isnan(ref[2, 3])
    mask = ~np.isnan(ref)
    assert np.max(np.abs(out[mask] - ref[mask])) <= 1e-14


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (2, 3, 1), (63, 65, 17), (127, 129, 200),
                                   (300, 1, 64), (1, 300, 64), (64, 64, 64), (513, 257, 96)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_gemm_edge_sizes_vs_oracle(cuda, port, m, n, k, ta, tb):
    A = oracle.uniform(m * 7 + n, m if ta == "N" else k, k if ta == "N" else m)
    B = oracle.uniform(n * 5 + k, k if tb == "N" else n, n if tb == "N" else k)
    C = oracle.uniform(k * 3 + m, m, n)
    out = fg.dgemm(ta, tb, -0.75, A, B, 1.5, C.copy(order="F"))
    ref = port.dgemm(ta, tb, -0.75, A, B, 1.5, C.copy(order="F"))
    assert rel(out, ref) <= GEMM_TOL


@pytest.mark.parametrize("m,n,k", [(1000, 900, 64), (1100, 700, 255), (640, 2048, 16)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_gemm_short_k_many_tiles_vs_oracle(cuda, port, m, n, k, ta, tb):
    # more 64x64 tiles than SMs and a short K (the LU's trailing-update
    # shape), ragged edges in m, n and k
    A = oracle.uniform(m + 3 * k, m if ta == "N" else k, k if ta == "N" else m)
    B = oracle.uniform(n + 5 * k, k if tb == "N" else n, n if tb == "N" else k)
    C = oracle.uniform(m + n, m, n)
    C[5, 7] = np.nan                     # beta*C is a multiply: NaN survives beta = 0
    out0 = fg.dgemm(ta, tb, 1.25, A, B, 0.0, C.copy(order="F"))
    assert np.isnan(out0[5, 7]) and np.isfinite(np.delete(out0.ravel(order="F"), 5 + 7 * m)).all()
    C[5, 7] = 0.25
    out = fg.dgemm(ta, tb, -0.75, A, B, 1.5, C.copy(order="F"))
    ref = port.dgemm(ta, tb, -0.75, A, B, 1.5, C.copy(order="F"))
    assert rel(out, ref) <= GEMM_TOL


def test_gemm_leading_dimension_views(cuda, port):
    # operands that are sub-blocks of larger arrays (ld > rows)
    big = oracle.uniform(11, 100, 90)
    A = big[3:40, 5:50]            # 37 x 45, ld = 100
    Bbig = oracle.uniform(12, 80, 70)
    B = Bbig[10:55, 0:33]          # 45 x 33, ld = 80
    Cbig = oracle.uniform(13, 60, 40)
    C = Cbig[1:38, 2:35]           # 37 x 33, ld = 60
    ref = port.dgemm("N", "N", 1.5, np.asfortranarray(A), np.asfortranarray(B), 0.5,
                     np.asfortranarray(C))
    # call dgemm_ directly on the strided views with their true leading dimensions
    import ctypes
    L = fg.lib()
    Cw = Cbig.copy(order="F")
    i = lambda v: ctypes.byref(ctypes.c_int(v))
    d = lambda v: ctypes.byref(ctypes.c_double(v))
    ptr = lambda arr, r, c: ctypes.cast(arr.ctypes.data + 8 * (r + c * arr.shape[0]),
                                        ctypes.POINTER(ctypes.c_double))
    L.dgemm_(b"N", b"N", i(37), i(33), i(45), d(1.5), ptr(big, 3, 5), i(100), ptr(Bbig, 10, 0),
             i(80), d(0.5), ptr(Cw, 1, 2), i(60))
    assert rel(Cw[1:38, 2:35], ref) <= GEMM_TOL
    untouched = np.ones_like(Cw, dtype=bool)
    untouched[1:38, 2:35] = False
    assert np.array_equal(Cw[untouched], Cbig[untouched])


def test_gemm_config1_full_size(cuda, port):
    # M=N=K=1024, alpha=1.5, beta=0.5, uniform[-1,1]: the GEMM workload config
    n = 1024
    A, B, C = oracle.uniform(101, n, n), oracle.uniform(102, n, n), oracle.uniform(103, n, n)
    out = fg.dgemm("N", "N", 1.5, A, B, 0.5, C.copy(order="F"))
    ref = port.dgemm("N", "N", 1.5, A, B, 0.5, C.copy(order="F"))
    assert rel(out, ref) <= GEMM_TOL, rel(out, ref)


def test_trsm_fixtures_host_api(cuda, golden):
    for i, (name, (m, n, side, uplo, ta, diag, alpha)) in enumerate(G.trsm_case_list()):
        A, B = G.trsm_inputs(i, m, n, side)
        out = fg.dtrsm(side, uplo, ta, diag, alpha, A, B.copy(order="F"))
        assert rel(out, golden[name]) <= TRSM_TOL, (name, rel(out, golden[name]))


@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("ta", "NT")
@pytest.mark.parametrize("diag", "UN")
@pytest.mark.parametrize("nvec", [37, 600])
def test_trsm_blocked_vs_oracle(cuda, port, side, uplo, ta, diag, nvec):
    # sizes that cross the 64-wide diagonal blocks; 37 vectors take the
    # warp-per-vector kernel, 600 the thread-per-vector kernel
    m, n = (200, nvec) if side == "L" else (nvec, 200)
    ka = m if side == "L" else n
    A = oracle.uniform(ka + 1, ka, ka)
    A[np.arange(ka), np.arange(ka)] += 2.0 + ka / 4.0
    B = oracle.uniform(ka + 2, m, n)
    out = fg.dtrsm(side, uplo, ta, diag, 1.5, A, B.copy(order="F"))
    ref = port.dtrsm(side, uplo, ta, diag, 1.5, A, B.copy(order="F"))
    assert rel(out, ref) <= TRSM_TOL


def test_trsm_device_api(cuda, port):
    import torch
    A = oracle.uniform(21, 130, 130)
    A[np.arange(130), np.arange(130)] += 40.0
    B = oracle.uniform(22, 130, 20)
    dA = fg.to_colmajor(torch.from_numpy(A).cuda())
    dB = fg.to_colmajor(torch.from_numpy(B).cuda())
    fg.dtrsm_dev("L", "U", "N", "N", 1.0, dA, dB)
    torch.cuda.synchronize()
    ref = port.dtrsm("L", "U", "N", "N", 1.0, A, B.copy(order="F"))
    assert rel(dB.cpu().numpy(), ref) <= TRSM_TOL


@pytest.mark.parametrize("n", [1, 2, 3, 4])
@pytest.mark.parametrize("tb", ["N", "T"])
def test_gemm_long_k_few_vectors_vs_oracle(cuda, port, n, tb):
    # op(A) = A with k >= 256, m*k >= 2^20 and n <= 4 runs the row-tile GEMV
    # (the residual and Krylov products of the refinement); m not a multiple
    # of the 16-row tile, a leading dimension larger than m
    m, k, lda = 1029, 1100, 1040
    Afull = oracle.uniform(91 + n, lda, k)
    A = np.asfortranarray(Afull[:m, :])
    B = oracle.uniform(92 + n, k if tb == "N" else n, n if tb == "N" else k)
    C = oracle.uniform(93 + n, m, n)
    out = fg.dgemm("N", tb, 1.5, A, B, -0.5, C.copy(order="F"))
    ref = port.dgemm("N", tb, 1.5, A, B, -0.5, C.copy(order="F"))
    assert rel(out, ref) <= GEMM_TOL, rel(out, ref)


def test_gemm_long_k_ld_view_device(cuda):
    import torch
    # device operands with ld > m: only the m x k view may be read
    m, k, lda = 2000, 3000, 2048
    g = torch.Generator(device=cuda)
    g.manual_seed(5)
    Abig = fg.to_colmajor(torch.rand((lda, k), generator=g, dtype=torch.float64, device=cuda) - 0.5)
    Abig[m:, :] = float("nan")
    A = Abig[:m, :]
    x = fg.to_colmajor(torch.rand((k, 1), generator=g, dtype=torch.float64, device=cuda))
    y = fg.colmajor_empty(m, 1, device=cuda)
    y.zero_()
    fg.dgemm_dev("N", "N", 1.0, A, x, 0.0, y)
    torch.cuda.synchronize()
    ref = A @ x
    assert torch.isfinite(y).all()
    assert ((y - ref).abs().max() / ref.abs().max()).item() <= GEMM_TOL
