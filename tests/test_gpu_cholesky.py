"""Cholesky (dpotrf_/dpotrs_/dposv_) and dsyrk_ on the GPU against the
reference's own results (tests/golden, made by the compiled FLENS shims).

Bars (flens/lapack/po/potrf.tcc, potrs.tcc, posv.tcc; cxxblas syrk):
* INFO identical to the reference's on every case, including the
  non-positive-definite ones (first failing column);
* the factor within 1e-12 normwise of the reference's, backward error
  ||A - L L^T|| / (n ||A|| eps) <= 10, the other triangle of A untouched;
* on failure, the factor of the leading INFO-1 columns and the stored failing
  pivot agree with the reference's;
* solves within 1e-12 normwise of the reference's;
* syrk within 1e-13 normwise on the triangle, the other triangle untouched.
"""
import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def tri(X, uplo):
    return np.tril(X) if uplo == "L" else np.triu(X)


def chol_backward_error(A0, F, uplo):
    n = A0.shape[0]
    L = np.tril(F) if uplo == "L" else np.triu(F).T
    R = np.tril(A0 - L @ L.T)
    return np.abs(R).sum(0).max() / (n * np.abs(A0).sum(0).max() * EPS)


def test_potrf_potrs_vs_reference(golden):
    for i, (name, (n, uplo, kind)) in enumerate(G.chol_case_list()):
        A0 = G.chol_input(i, n, kind)
        A = A0.copy(order="F")
        info = fg.dpotrf(uplo, A)
        ref = golden[name + "_A"]
        assert info == golden[name + "_info"][0], (name, info)
        other = np.triu(np.ones((n, n)), 1) if uplo == "L" else np.tril(np.ones((n, n)), -1)
        assert np.array_equal(A[other > 0], A0[other > 0]), name          # other triangle untouched
        if kind == "spd":
            assert oracle.normwise_rel(tri(A, uplo), tri(ref, uplo)) <= 1e-12, name
            assert chol_backward_error(A0, A, uplo) <= 10.0, name
            B = G.chol_rhs(i, n).copy(order="F")
            X, st = fg.dpotrs(uplo, A, B)
            assert st == 0
            assert oracle.normwise_rel(X, golden[name + "_X"]) <= 1e-12, name
        else:
            f = info - 1                                                  # failing column
            lead = tri(A, uplo)[:f, :f]
            assert oracle.normwise_rel(lead, tri(ref, uplo)[:f, :f]) <= 1e-12, name
            assert A[f, f] <= 0.0 and ref[f, f] <= 0.0
            assert abs(A[f, f] - ref[f, f]) <= 1e-12 * abs(ref[f, f]), name


def test_posv_reports_info_and_skips_solve(port):
    n = 70
    for uplo in "LU":
        A0 = G.chol_input(3, n, "spd")
        B0 = G.chol_rhs(3, n)
        A, B = A0.copy(order="F"), B0.copy(order="F")
        assert fg.dposv(uplo, A, B) == 0
        Ar, Br = A0.copy(order="F"), B0.copy(order="F")
        assert port.dposv(uplo, Ar, Br) == 0
        assert oracle.normwise_rel(B, Br) <= 1e-12
        An = G.chol_input(4, n, "notpd")
        A, B = An.copy(order="F"), B0.copy(order="F")
        assert fg.dposv(uplo, A, B) == n // 2 + 1      # LAPACK DPOSV semantics
        assert np.array_equal(B, B0)                   # no solve (posv.tcc:58-64)


def test_syrk_vs_reference(golden):
    for i, (name, (n, k, uplo, tr, a, b)) in enumerate(G.syrk_case_list()):
        A, C0 = G.syrk_inputs(i, n, k, tr)
        C = fg.dsyrk(uplo, tr, a, A, b, C0.copy(order="F"))
        want = golden[name]
        if n == 0:
            continue
        mask = np.tril(np.ones((n, n))) if uplo == "L" else np.triu(np.ones((n, n)))
        assert np.array_equal(C[mask == 0], C0[mask == 0]), name
        assert oracle.normwise_rel(C * mask, want * mask) <= 1e-13, name


@pytest.mark.parametrize("n", [1, 64, 65, 300, 1000])
def test_device_potrf_posv(cuda, port, n):
    import torch
    G0 = oracle.uniform(np.random.default_rng(n), n, n)
    A0 = np.asfortranarray(G0 @ G0.T / n + np.eye(n))
    B0 = oracle.uniform(np.random.default_rng(n + 1), n, 2)
    for uplo in "lu":                                   # the device API takes either case
        A = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
        B = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        info = torch.full((1,), -5, dtype=torch.int32, device=cuda)
        fg.dposv_dev(uplo, A, B, info)
        assert int(info.item()) == 0
        Ar, Br = A0.copy(order="F"), B0.copy(order="F")
        assert port.dposv(uplo.upper(), Ar, Br) == 0
        assert oracle.normwise_rel(B.cpu().numpy(), Br) <= 1e-12
        assert chol_backward_error(A0, A.cpu().numpy(), uplo.upper()) <= 10.0


def test_device_syrk_large(cuda, port):
    import torch
    n, k = 700, 300
    rng = np.random.default_rng(5)
    for uplo in "LU":
        for tr in "NT":
            A = oracle.uniform(rng, n if tr == "N" else k, k if tr == "N" else n)
            C0 = oracle.uniform(rng, n, n)
            Cd = fg.to_colmajor(torch.from_numpy(C0).to(cuda))
            fg.dsyrk_dev(uplo, tr, -0.5, fg.to_colmajor(torch.from_numpy(A).to(cuda)), 2.0, Cd)
            want = port.dsyrk(uplo, tr, -0.5, A, 2.0, C0.copy(order="F"))
            mask = np.tril(np.ones((n, n))) if uplo == "L" else np.triu(np.ones((n, n)))
            got = Cd.cpu().numpy()
            assert np.array_equal(got[mask == 0], C0[mask == 0])
            assert oracle.normwise_rel(got * mask, want * mask) <= 1e-13


@pytest.mark.slow
def test_potrf_full_size(cuda):
    """n = 8192 SPD (G G^T / n + I, torch-seeded G): backward error and a
    solve against a known solution."""
    import torch
    n = 8192
    g = torch.Generator(device=cuda).manual_seed(81)
    Gm = torch.rand((n, n), generator=g, dtype=torch.float64, device=cuda) * 2 - 1
    A0 = (Gm @ Gm.T) / n + torch.eye(n, dtype=torch.float64, device=cuda)
    del Gm
    x = torch.rand((n, 1), generator=g, dtype=torch.float64, device=cuda) * 2 - 1
    b = A0 @ x
    A = fg.to_colmajor(A0.clone())
    B = b.clone()
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dposv_dev("L", A, B, info)
    assert int(info.item()) == 0
    L = torch.tril(A)
    R = torch.tril(A0 - L @ L.T)
    be = (R.abs().sum(0).max() / (n * A0.abs().sum(0).max() * EPS)).item()
    assert be <= 10.0, be
    assert ((B - x).abs().max() / x.abs().max()).item() <= 1e-10
