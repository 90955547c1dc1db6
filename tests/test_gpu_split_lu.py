"""Precision form: the FP64-accurate LU whose trailing updates beyond each
outer block run through the split GEMM (flens_gb300_dgetrf_split), and the
mixed solve built on it (flens_gb300_dgesv_mixed, precision 4).

Bars (in the asserts): the trf bar of the plain form, backward error
||PA - LU||_1 / (n ||A||_1 eps) <= 10; pivots and INFO identical to the
reference's (the oracle restatement, pinned to the compiled reference) on
inputs whose column maxima are separated by much more than rounding; at
n = 8192 the reference's own pivots and diag(U) within 1e-12.  The solve
reaches the normwise backward error <= 10 n eps64 at kappa = 1e10, where FP32
factors cannot (kappa u32 ~ 600), in at most 3 refinement steps.
"""
import os

import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
BERR_TOL = 10.0


def split_lu(cuda, A0, outer_nb):
    import torch
    m, n = A0.shape
    dA = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    ipiv = torch.zeros(max(1, min(m, n)), dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_split_dev(dA, ipiv, info, outer_nb)
    fg.sync()
    return dA.cpu().numpy(), ipiv.cpu().numpy()[:min(m, n)], int(info.item())


@pytest.mark.parametrize("m,n", [(300, 300), (700, 700), (1000, 600), (600, 1000), (1100, 1100),
                                 (129, 700), (700, 129)])
@pytest.mark.parametrize("outer_nb", [128, 512])
def test_split_lu_vs_oracle(cuda, port, m, n, outer_nb):
    A0 = oracle.uniform(m * 17 + n, m, n)
    LU, piv, info = split_lu(cuda, A0, outer_nb)
    LUr = A0.copy(order="F")
    pivr, infor = port.dgetrf(LUr)
    assert info == infor
    assert np.array_equal(piv, pivr)
    assert oracle.lu_backward_error(A0, LU, piv) <= BERR_TOL
    # the factors themselves: FP64-accurate, so close to the reference's
    assert oracle.normwise_rel(LU, LUr) <= 1e-10


@pytest.mark.parametrize("outer_nb", [64, 192, 0])
def test_split_lu_outer_blocks(cuda, port, outer_nb):
    n = 777
    A0 = oracle.uniform(4242, n, n)
    A0[np.arange(n), np.arange(n)] += n / 4.0
    LU, piv, info = split_lu(cuda, A0, outer_nb)
    LUr = A0.copy(order="F")
    pivr, infor = port.dgetrf(LUr)
    assert info == infor == 0
    assert np.array_equal(piv, pivr)
    assert oracle.lu_backward_error(A0, LU, piv) <= BERR_TOL
    assert oracle.normwise_rel(LU, LUr) <= 1e-13


def test_split_lu_singular_info(cuda, port):
    # a zero column beyond the first outer block stays exactly zero through
    # the split updates (zero digits), so INFO is the reference's
    n = 400
    A0 = oracle.uniform(99, n, n)
    A0[:, 300] = 0.0
    LU, piv, info = split_lu(cuda, A0, 128)
    LUr = A0.copy(order="F")
    pivr, infor = port.dgetrf(LUr)
    assert info == infor == 301
    assert np.array_equal(piv, pivr)


@pytest.mark.parametrize("nrhs", [1, 64])
def test_mixed_split_kappa_1e10(cuda, nrhs):
    from test_gpu_mixed import backward_error, dgesv_mixed, make_system
    n, kappa = 1024, 1e10
    A, b, x = make_system(cuda, n, kappa, nrhs, 21)
    st, X, it, be, inf = dgesv_mixed(A, b, "split", "auto")
    assert st == 0 and inf == 0, (st, fg.last_error(), it, be)
    assert it <= 3, it
    assert be <= 10 * n * EPS
    assert backward_error(A, X, b) <= 10 * n * EPS
    fwd = ((X - x).abs().max() / x.abs().max()).item()
    assert fwd <= kappa * 1e3 * EPS, fwd


def test_mixed_split_singular_info(cuda):
    from test_gpu_mixed import dgesv_mixed, make_system
    n = 700
    A, b, x = make_system(cuda, n, 10.0, 1, 22)
    A[:, 600] = 0.0
    st, X, it, be, inf = dgesv_mixed(A, b, "split", "auto")
    assert st == 0 and inf == 601


@pytest.mark.slow
def test_split_lu_full_size(cuda):
    """n=8192 shifted LU (the plain form's workload) through the split LU:
    backward error, the reference's pivots and diag(U)."""
    import torch
    n = G.LARGE_N
    A0 = G.large_lu_input()
    dA0 = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    dA = fg.to_colmajor(dA0.clone())
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_split_dev(dA, ipiv, info)
    fg.sync()
    assert int(info.item()) == 0
    piv = ipiv.cpu().numpy()
    path = os.path.join(G.HERE, "reference_lu8192.npz")
    ref = np.load(path)
    assert np.array_equal(piv, ref["piv"])
    d_gpu = torch.diagonal(dA).cpu().numpy()
    assert np.max(np.abs(d_gpu - ref["diagU"]) / np.abs(ref["diagU"])) <= 1e-12
    L = torch.tril(dA, -1) + torch.eye(n, dtype=torch.float64, device=cuda)
    U = torch.triu(dA)
    P = torch.arange(n, device=cuda)
    for i, p in enumerate(piv.tolist()):
        if p - 1 != i:
            P[[i, p - 1]] = P[[p - 1, i]]
    R = dA0[P] - L @ U
    berr = (R.abs().sum(0).max() / (n * dA0.abs().sum(0).max() * EPS)).item()
    assert berr <= BERR_TOL, berr
