"""Pins the CPU oracle (oracle/flens_oracle.c) to the reference.

1. Against the committed fixtures made by running the reference's own
   dgemm_/dtrsm_/dgetrf_/dgetrs_/dgesv_ (tests/golden/make_golden.py): the
   restatement must be BITWISE identical on every case.
2. Live against oracle/_ref (the reference shims compiled from source) on
   extra random cases, when that library was built in this checkout.
"""
import os

import numpy as np
import pytest

import make_golden as G
import oracle


def test_gemm_fixtures_bitwise(golden, port):
    for i, (name, (m, n, k, ta, tb, a, b)) in enumerate(G.gemm_case_list()):
        A, B, C = G.gemm_inputs(i, m, n, k, ta, tb)
        out = port.dgemm(ta, tb, a, A, B, b, C.copy(order="F"))
        assert np.array_equal(out, golden[name], equal_nan=True), name


def test_trsm_fixtures_bitwise(golden, port):
    for i, (name, (m, n, side, uplo, ta, diag, alpha)) in enumerate(G.trsm_case_list()):
        A, B = G.trsm_inputs(i, m, n, side)
        out = port.dtrsm(side, uplo, ta, diag, alpha, A, B.copy(order="F"))
        assert np.array_equal(out, golden[name]), name


def test_lu_fixtures_bitwise(golden, port):
    for i, (name, (m, n, kind)) in enumerate(G.lu_case_list()):
        LU = G.lu_input(i, m, n, kind)
        piv, info = port.dgetrf(LU)
        assert np.array_equal(LU, golden[name + "_LU"]), name
        assert np.array_equal(piv, golden[name + "_piv"]), name
        assert info == golden[name + "_info"][0], name
        if m == n:
            Bm = G.lu_rhs(i, n)
            for t in "NT":
                X = port.dgetrs(t, LU, piv, Bm.copy(order="F"))
                assert np.array_equal(X, golden[name + f"_X{t}"]), (name, t)


def test_singular_info(golden, port):
    LU = G.singular_input()
    piv, info = port.dgetrf(LU)
    assert info == golden["sing_info"][0] == 3
    assert np.array_equal(piv, golden["sing_piv"])
    assert np.array_equal(LU, golden["sing_LU"])


def test_baby_problem_known_answer(golden, port):
    # flens/examples/lapack-gesv.cc: x = (1, 9, 9, 9), piv = (2, 3, 4, 4)
    A, b = G.baby_problem()
    piv, info = port.dgesv(A, b)
    assert info == 0
    assert np.array_equal(piv, [2, 3, 4, 4])
    assert np.allclose(b[:, 0], [1, 9, 9, 9], rtol=0, atol=1e-13)
    assert np.array_equal(b, golden["baby_x"])
    assert np.array_equal(piv, golden["baby_piv"])
    assert np.array_equal(A, golden["baby_LU"])


def test_syrk_fixtures_bitwise(golden, port):
    for i, (name, (n, k, uplo, tr, a, b)) in enumerate(G.syrk_case_list()):
        A, C = G.syrk_inputs(i, n, k, tr)
        out = port.dsyrk(uplo, tr, a, A, b, C.copy(order="F"))
        assert np.array_equal(out, golden[name]), name


def test_trmm_symm_syr2k_fixtures_bitwise(golden, port):
    for i, (name, (m, n, side, uplo, ta, diag, alpha)) in enumerate(G.trmm_case_list()):
        A, B = G.trmm_inputs(i, m, n, side)
        out = port.dtrmm(side, uplo, ta, diag, alpha, A, B.copy(order="F"))
        assert np.array_equal(out, golden[name]), name
    for i, (name, (m, n, side, uplo, a, b)) in enumerate(G.symm_case_list()):
        A, B, C = G.symm_inputs(i, m, n, side)
        assert np.array_equal(port.dsymm(side, uplo, a, A, B, b, C.copy(order="F")), golden[name]), name
    for i, (name, (n, k, uplo, tr, a, b)) in enumerate(G.syr2k_case_list()):
        A, B, C = G.syr2k_inputs(i, n, k, tr)
        assert np.array_equal(port.dsyr2k(uplo, tr, a, A, B, b, C.copy(order="F")), golden[name]), name


def test_trtri_getri_fixtures_bitwise(golden, port):
    for i, (name, (n, uplo, diag)) in enumerate(G.tri_case_list()):
        A = G.tri_input(i, n)
        assert port.dtrtri(uplo, diag, A) == 0
        assert np.array_equal(A, golden[name]), name
    for i, (name, n) in enumerate(G.getri_case_list()):
        LU = G.getri_input(i, n)
        piv, info = port.dgetrf(LU)
        assert port.dgetri(LU, piv) == 0
        assert np.array_equal(LU, golden[name]), name
    # a zero diagonal element: the routine's INFO, A untouched (tr/tri.tcc)
    A = G.tri_input(0, 10)
    A[3, 3] = 0.0
    A0 = A.copy()
    assert port.dtrtri("U", "N", A) == 4 and np.array_equal(A, A0)


def test_refinement_condition_equilibration_bitwise(golden, port):
    """gecon, gerfs, geequ, laqge, gesvx against the reference's results.  The
    reference's dgesvx_ returns EQUED = 'N' even after equilibrating (svx
    takes equed by value, flens/lapack/ge/svx.tcc): only the results are
    compared, EQUED is checked against what the scaled A shows."""
    for i, (name, n) in enumerate(G.refine_case_list()):
        A, Ae, B = G.refine_inputs(i, n)
        LU = A.copy(order="F")
        piv, _ = port.dgetrf(LU)
        rc = [port.dgecon(nm, LU, port.dlange("1" if nm != "I" else "I", A)) for nm in ("1", "I")]
        assert all(st == 0 for _, st in rc), name
        assert np.array_equal(np.array([v for v, _ in rc]), golden[name + "_rcond"]), name
        for tr in "NT":
            X = B.copy(order="F")
            port.dgetrs(tr, LU, piv, X)
            X[0, :] += 1e-8
            ferr, berr = port.dgerfs(tr, A, LU, piv, B, X)
            assert np.array_equal(X, golden[name + f"_rfs{tr}_X"]), (name, tr)
            assert np.array_equal(ferr, golden[name + f"_rfs{tr}_ferr"]), (name, tr)
            assert np.array_equal(berr, golden[name + f"_rfs{tr}_berr"]), (name, tr)
        r, c, rcnd, ccnd, amax, info = port.dgeequ(Ae)
        assert np.array_equal(np.concatenate([r, c, [rcnd, ccnd, amax, info]]), golden[name + "_equ"])
        for fact in "NE":
            for tr in "NT":
                Aw, Bw = Ae.copy(order="F"), B.copy(order="F")
                AF, Xw = np.zeros((n, n), order="F"), np.zeros((n, 3), order="F")
                pv = np.zeros(n, dtype=np.int32)
                info, eq, rcn, fe, be, g = port.dgesvx(fact, tr, Aw, AF, pv, "N", np.zeros(n),
                                                       np.zeros(n), Bw, Xw)
                k = name + f"_svx{fact}{tr}"
                assert np.array_equal(Xw, golden[k + "_X"]), k
                assert np.array_equal(AF, golden[k + "_AF"]), k
                assert np.array_equal(Aw, golden[k + "_A"]), k
                assert np.array_equal(np.concatenate([[info, rcn, g], fe, be]), golden[k + "_s"]), k
                assert (eq == "N") == np.array_equal(Aw, Ae), k
    A = G.singular_input()
    n = A.shape[0]
    AF, X = np.zeros((n, n), order="F"), np.zeros((n, 1), order="F")
    info, eq, rcn, fe, be, g = port.dgesvx("N", "N", A, AF, np.zeros(n, dtype=np.int32), "N",
                                           np.zeros(n), np.zeros(n), G.U(7778, n, 1), X)
    assert np.array_equal(np.array([info, rcn, g]), golden["svx_sing_s"]) and info == 3


def test_cholesky_fixtures_bitwise(golden, port):
    for i, (name, (n, uplo, kind)) in enumerate(G.chol_case_list()):
        A = G.chol_input(i, n, kind)
        info = port.dpotrf(uplo, A)
        assert info == golden[name + "_info"][0], name
        assert np.array_equal(A, golden[name + "_A"]), name
        if kind == "notpd":
            assert info == n // 2 + 1, name
        else:
            assert info == 0, name
            X = port.dpotrs(uplo, A, G.chol_rhs(i, n).copy(order="F"))
            assert np.array_equal(X, golden[name + "_X"]), name


def test_iamax_first_max_and_nan():
    p = oracle.Port()
    assert p.idamax([1.0, -3.0, 3.0, 2.0]) == 1          # first maximum wins
    assert p.idamax([float("nan"), 5.0, 1.0]) == 0       # NaN at 0: nothing compares greater
    assert p.idamax([1.0, float("nan"), 5.0]) == 2       # a later NaN never wins
    assert p.idamax([]) == -1


def test_large_pivot_fixture_consistent():
    path = os.path.join(G.HERE, "reference_lu8192.npz")
    if not os.path.exists(path):
        pytest.skip("n=8192 fixture not generated")
    d = np.load(path)
    n, seed, info, nonid = d["meta"].tolist()
    assert (n, seed) == (G.LARGE_N, G.LARGE_SEED)
    assert info == 0
    assert nonid == int(np.count_nonzero(d["piv"] != np.arange(1, n + 1)))


@pytest.mark.skipif(not oracle.reference_available(), reason="oracle/_ref not built here")
def test_port_equals_reference_live():
    R, P = oracle.Reference(), oracle.Port()
    rng = np.random.default_rng(99)
    for (m, n, k) in [(5, 9, 13), (40, 41, 42)]:
        for ta in "NT":
            for tb in "NT":
                A = oracle.uniform(rng, m if ta == "N" else k, k if ta == "N" else m)
                B = oracle.uniform(rng, k if tb == "N" else n, n if tb == "N" else k)
                C = oracle.uniform(rng, m, n)
                assert np.array_equal(P.dgemm(ta, tb, 0.3, A, B, -1.1, C.copy(order="F")),
                                      R.dgemm(ta, tb, 0.3, A, B, -1.1, C.copy(order="F")))
    for (m, n) in [(90, 90), (150, 120), (70, 200)]:
        A = oracle.uniform(rng, m, n)
        a1, a2 = A.copy(order="F"), A.copy(order="F")
        p1, i1 = P.dgetrf(a1)
        p2, i2 = R.dgetrf(a2)
        assert np.array_equal(a1, a2) and np.array_equal(p1, p2) and i1 == i2
    for n in (70, 150):
        G0 = oracle.uniform(rng, n, n)
        A = np.asfortranarray(G0 @ G0.T / n + np.eye(n))
        for uplo in "LU":
            a1, a2 = A.copy(order="F"), A.copy(order="F")
            assert P.dpotrf(uplo, a1) == R.dpotrf(uplo, a2) == 0
            assert np.array_equal(a1, a2)
            B = oracle.uniform(rng, n, 2)
            b1 = P.dpotrs(uplo, a1, B.copy(order="F"))
            b2, _ = R.dpotrs(uplo, a2, B.copy(order="F"))
            assert np.array_equal(b1, b2)
    # the reference's dposv_ drops posv's INFO (posv.cc:50); its C++ posv
    # returns it, as the restatement does
    A = np.asfortranarray(np.eye(6))
    A[2, 2] = -1.0
    assert R.dposv("L", A.copy(order="F"), np.ones((6, 1), order="F")) == 0
    assert P.dposv("L", A.copy(order="F"), np.ones((6, 1), order="F")) == 3
