"""dtrtri_ and dgetri_ on the GPU against the reference's own results
(tests/golden, from the compiled FLENS shims) and, at full size, against the
identity.

Bars: normwise relative error <= 1e-12 against the reference's inverse (the
inputs are diagonally dominant, so the inverses are well conditioned); the
other triangle of a triangular inverse untouched, a unit diagonal not
written; INFO for an exactly zero diagonal element with A untouched (LAPACK
semantics); ||A inv(A) - I|| / (n ||A|| ||inv(A)|| eps) small at full size.
"""
import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def test_trtri_vs_reference(golden):
    for i, (name, (n, uplo, diag)) in enumerate(G.tri_case_list()):
        A0 = G.tri_input(i, n)
        A = A0.copy(order="F")
        assert fg.dtrtri(uplo, diag, A) == 0, name
        want = golden[name]
        mask = np.triu(np.ones((n, n))) if uplo == "U" else np.tril(np.ones((n, n)))
        if diag == "U":
            np.fill_diagonal(mask, 0)
        assert np.array_equal(A[mask == 0], A0[mask == 0]), name        # untouched part
        assert oracle.normwise_rel(A * mask, want * mask) <= 1e-12, name


def test_getri_vs_reference(golden, port):
    for i, (name, n) in enumerate(G.getri_case_list()):
        LU = G.getri_input(i, n)
        piv, info = port.dgetrf(LU)
        assert info == 0
        assert fg.dgetri(LU, piv) == 0
        assert oracle.normwise_rel(LU, golden[name]) <= 1e-12, name


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("diag", "NU")
def test_trtri_outer_blocks_vs_oracle(port, uplo, diag):
    # n > 512: outer blocks of 512 around the 64-column inner algorithm
    n = 1100
    A0 = G.tri_input(3, n)
    A = A0.copy(order="F")
    assert fg.dtrtri(uplo, diag, A) == 0
    R = A0.copy(order="F")
    port.dtrtri(uplo, diag, R)
    mask = np.triu(np.ones((n, n))) if uplo == "U" else np.tril(np.ones((n, n)))
    if diag == "U":
        np.fill_diagonal(mask, 0)
    assert np.array_equal(A[mask == 0], A0[mask == 0])
    assert oracle.normwise_rel(A * mask, R * mask) <= 1e-12


def test_getri_outer_blocks_vs_oracle(port):
    n = 1100
    LU = G.getri_input(4, n)
    piv, info = port.dgetrf(LU)
    assert info == 0
    R = LU.copy(order="F")
    port.dgetri(R, piv)
    assert fg.dgetri(LU, piv) == 0
    assert oracle.normwise_rel(LU, R) <= 1e-12


def test_zero_pivot_info():
    A = G.tri_input(0, 70)
    A[40, 40] = 0.0
    A0 = A.copy()
    assert fg.dtrtri("U", "N", A) == 41
    assert np.array_equal(A, A0)
    # a singular U in dgetri: INFO and A left as the factors
    LU = G.getri_input(2, 70)                           # read as factors: U(11,11) = 0
    LU[10, 10] = 0.0
    LU0 = LU.copy()
    assert fg.dgetri(LU, np.arange(1, 71, dtype=np.int32)) == 11
    assert np.array_equal(LU, LU0)


@pytest.mark.parametrize("n", [300, 1000])
def test_device_getri_identity(cuda, n):
    import torch
    A0 = G.getri_input(7, n)
    A = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_dev(A, ipiv, info)
    assert int(info.item()) == 0
    st = fg.lib().flens_gb300_dgetri(n, A.data_ptr(), n, ipiv.data_ptr(), info.data_ptr(), None)
    assert st == 0 and int(info.item()) == 0
    X = A.cpu().numpy()
    R = A0 @ X - np.eye(n)
    nrm = lambda M: np.abs(M).sum(0).max()
    assert nrm(R) / (n * nrm(A0) * nrm(X) * EPS) <= 1.0


@pytest.mark.slow
def test_getri_full_size(cuda):
    """n = 8192 (uniform + n/4 I): inverse through the device entry points."""
    import torch
    n = 8192
    g = torch.Generator(device=cuda).manual_seed(91)
    A0 = torch.rand((n, n), generator=g, dtype=torch.float64, device=cuda) * 2 - 1
    A0.diagonal().add_(n / 4.0)
    A0 = A0.t()
    A = fg.to_colmajor(A0.clone())
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_dev(A, ipiv, info)
    st = fg.lib().flens_gb300_dgetri(n, A.data_ptr(), n, ipiv.data_ptr(), info.data_ptr(), None)
    assert st == 0 and int(info.item()) == 0
    R = A0 @ A - torch.eye(n, dtype=torch.float64, device=cuda)
    nrm = lambda M: M.abs().sum(0).max().item()
    assert nrm(R) / (n * nrm(A0) * nrm(A) * EPS) <= 1.0
