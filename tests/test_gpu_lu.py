"""GPU parity for dgetrf / dgetrs / dgesv through the C ABI.

Bars: backward error ||PA - LU||_1 / (n ||A||_1 eps) <= 10 (the project's trf
parity bar), identical pivot vectors and INFO on the reference fixtures (inputs whose
column maxima are well separated, and unshifted uniform inputs at these small
sizes), solutions within 1e-12 normwise of the reference's.
"""
import os

import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu

BERR_TOL = 10.0
SOLVE_TOL = 1e-12


def test_lu_fixtures_host_api(cuda, golden):
    for i, (name, (m, n, kind)) in enumerate(G.lu_case_list()):
        A0 = G.lu_input(i, m, n, kind)
        LU = A0.copy(order="F")
        piv, info = fg.dgetrf(LU)
        assert info == golden[name + "_info"][0], name
        assert np.array_equal(piv, golden[name + "_piv"]), (name, piv, golden[name + "_piv"])
        berr = oracle.lu_backward_error(A0, LU, piv)
        assert berr <= BERR_TOL, (name, berr)
        assert oracle.normwise_rel(LU, golden[name + "_LU"]) <= 1e-12, name
        if m == n:
            Bm = G.lu_rhs(i, n)
            for t in "NT":
                X, inf2 = fg.dgetrs(t, LU, piv, Bm.copy(order="F"))
                assert inf2 == 0
                assert oracle.normwise_rel(X, golden[name + f"_X{t}"]) <= SOLVE_TOL, (name, t)


def test_baby_problem(cuda, golden):
    # flens/examples/lapack-gesv.cc: x = (1, 9, 9, 9), piv = (2, 3, 4, 4)
    A, b = G.baby_problem()
    piv, info = fg.dgesv(A, b)
    assert info == 0
    assert np.array_equal(piv, golden["baby_piv"]) and np.array_equal(piv, [2, 3, 4, 4])
    assert np.allclose(b[:, 0], [1, 9, 9, 9], rtol=0, atol=1e-13)
    assert oracle.normwise_rel(A, golden["baby_LU"]) <= 1e-14


def test_singular_info(cuda, golden):
    A0 = G.singular_input()
    LU = A0.copy(order="F")
    piv, info = fg.dgetrf(LU)
    assert info == golden["sing_info"][0] == 3
    assert np.array_equal(piv, golden["sing_piv"])
    # dgesv: factorisation done, no solve (flens/lapack/ge/sv.tcc:70-75)
    A1 = A0.copy(order="F")
    b = oracle.uniform(5, 12, 2)
    b0 = b.copy()
    piv2, info2 = fg.dgesv(A1, b)
    assert info2 == 3 and np.array_equal(b, b0)


@pytest.mark.parametrize("m,n", [(1, 5), (5, 1), (3, 3), (63, 63), (65, 65), (127, 129),
                                 (129, 127), (200, 64), (64, 200), (257, 257), (1000, 70),
                                 (70, 1000)])
def test_lu_sizes_vs_oracle(cuda, port, m, n):
    A0 = oracle.uniform(m * 31 + n, m, n)
    LU = A0.copy(order="F")
    piv, info = fg.dgetrf(LU)
    LUr = A0.copy(order="F")
    pivr, infor = port.dgetrf(LUr)
    assert info == infor
    assert np.array_equal(piv, pivr)
    assert oracle.lu_backward_error(A0, LU, piv) <= BERR_TOL


@pytest.mark.parametrize("nrhs", [1, 2, 15, 16])
@pytest.mark.parametrize("trans", "NT")
def test_getrs_nrhs_grid(cuda, port, nrhs, trans):
    n = 150
    A0 = oracle.uniform(77, n, n)
    LU = A0.copy(order="F")
    piv, _ = port.dgetrf(LU)
    B = oracle.uniform(78 + nrhs, n, nrhs)
    X, info = fg.dgetrs(trans, LU, piv, B.copy(order="F"))
    Xr = port.dgetrs(trans, LU, piv, B.copy(order="F"))
    assert info == 0
    assert oracle.normwise_rel(X, Xr) <= SOLVE_TOL


def test_nan_pivot_rule(cuda, port):
    # a NaN on the diagonal: iamax keeps the first element (no row swap)
    A0 = oracle.uniform(5, 6, 6)
    A0[0, 0] = np.nan
    LU = A0.copy(order="F")
    piv, _ = fg.dgetrf(LU)
    LUr = A0.copy(order="F")
    pivr, _ = port.dgetrf(LUr)
    assert piv[0] == pivr[0] == 1


def test_device_api_gesv(cuda, port):
    import torch
    n, nrhs = 300, 4
    A0 = oracle.uniform(41, n, n)
    B0 = oracle.uniform(42, n, nrhs)
    dA = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    dB = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgesv_dev(dA, ipiv, dB, info)
    fg.sync()
    A1, B1 = A0.copy(order="F"), B0.copy(order="F")
    pivr, infor = port.dgesv(A1, B1)
    assert int(info.item()) == infor == 0
    assert np.array_equal(ipiv.cpu().numpy(), pivr)
    assert oracle.normwise_rel(dB.cpu().numpy(), B1) <= SOLVE_TOL


def test_config2_full_size(cuda):
    """n=8192 shifted LU + solve: backward error, pivots vs the reference run,
    forward error against x_true."""
    import torch
    n = G.LARGE_N
    A0 = G.large_lu_input()
    rng = np.random.default_rng(5)
    x_true = rng.uniform(-1.0, 1.0, size=(n, 1))
    dA0 = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    dA = fg.to_colmajor(dA0.clone())
    db = fg.to_colmajor(dA0 @ torch.from_numpy(x_true).to(cuda))
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_dev(dA, ipiv, info)
    fg.dgetrs_dev("N", dA, ipiv, db)
    fg.sync()
    assert int(info.item()) == 0
    piv = ipiv.cpu().numpy()
    path = os.path.join(G.HERE, "reference_lu8192.npz")
    if os.path.exists(path):
        ref = np.load(path)
        assert np.array_equal(piv, ref["piv"])
        d_gpu = torch.diagonal(dA).cpu().numpy()
        assert np.max(np.abs(d_gpu - ref["diagU"]) / np.abs(ref["diagU"])) <= 1e-12
    else:
        assert np.array_equal(piv, np.arange(1, n + 1))
    # backward error of the factorisation, computed on the GPU in FP64
    L = torch.tril(dA, -1) + torch.eye(n, dtype=torch.float64, device=cuda)
    U = torch.triu(dA)
    P = torch.arange(n, device=cuda)
    for i, p in enumerate(piv.tolist()):
        if p - 1 != i:
            P[[i, p - 1]] = P[[p - 1, i]]
    R = dA0[P] - L @ U
    eps = np.finfo(np.float64).eps
    berr = (R.abs().sum(0).max() / (n * dA0.abs().sum(0).max() * eps)).item()
    assert berr <= BERR_TOL, berr
    x = db.cpu().numpy()
    fwd = np.abs(x - x_true).max() / np.abs(x_true).max()
    assert fwd <= 1e-12, fwd


def _unshifted_case(n):
    path = os.path.join(G.HERE, "reference_lu_unshifted.npz")
    ref = np.load(path)
    _, seed, info = (int(v) for v in ref[f"n{n}_meta"])
    return (oracle.splitmix_uniform(seed, n, n), ref[f"n{n}_piv"], info, ref[f"n{n}_gap"],
            ref[f"n{n}_diagU"])


def _check_unshifted(cuda, n, dA0, dA, piv, info, ref_piv, ref_info, gap, ref_diag):
    import torch
    # pivots entry by entry on every pivot search whose two largest |candidates|
    # differ by more than 1e-10 relative (flens/lapack/ge/tf2.tcc:101-108,
    # cxxblas/level1/iamax.tcc:50-57); the fixture's smallest gap is ~1e-6, so
    # this is every column
    sep = gap > 1e-10
    assert sep.mean() > 0.99
    bad = np.nonzero((piv != ref_piv) & sep)[0]
    assert bad.size == 0, (bad[:10], piv[bad[:10]], ref_piv[bad[:10]])
    assert info == ref_info == 0
    assert np.count_nonzero(piv != np.arange(1, n + 1)) > 0.9 * n      # it really pivots
    d = torch.diagonal(dA).cpu().numpy()
    assert np.max(np.abs(d - ref_diag)) / np.max(np.abs(ref_diag)) <= 1e-9
    # backward error of the factorisation, on the GPU in FP64
    L = torch.tril(dA, -1) + torch.eye(n, dtype=torch.float64, device=cuda)
    U = torch.triu(dA)
    P = np.arange(n)
    for i, p in enumerate(piv.tolist()):
        if p - 1 != i:
            P[[i, p - 1]] = P[[p - 1, i]]
    R = dA0[torch.from_numpy(P).to(cuda)] - L @ U
    eps = np.finfo(np.float64).eps
    berr = (R.abs().sum(0).max() / (n * dA0.abs().sum(0).max() * eps)).item()
    assert berr <= BERR_TOL, berr


@pytest.mark.parametrize("n", [2048, 4096])
def test_pivots_unshifted_at_scale(cuda, n):
    """Unshifted uniform[-1,1) LU at n = 2048 and 4096 (about n interchanges)
    against the reference's own pivots and diag(U)."""
    import torch
    A0, ref_piv, ref_info, gap, ref_diag = _unshifted_case(n)
    dA0 = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    dA = fg.to_colmajor(dA0.clone())
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_dev(dA, ipiv, info)
    fg.sync()
    _check_unshifted(cuda, n, dA0, dA, ipiv.cpu().numpy(), int(info.item()), ref_piv, ref_info,
                     gap, ref_diag)


def test_split_lu_pivots_unshifted_n2048(cuda):
    """The FP64-accurate split-update LU on the same n = 2048 unshifted input."""
    import torch
    n = 2048
    A0, ref_piv, ref_info, gap, ref_diag = _unshifted_case(n)
    dA0 = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    dA = fg.to_colmajor(dA0.clone())
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_split_dev(dA, ipiv, info, 512)
    fg.sync()
    _check_unshifted(cuda, n, dA0, dA, ipiv.cpu().numpy(), int(info.item()), ref_piv, ref_info,
                     gap, ref_diag)
