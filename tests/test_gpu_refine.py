"""Refinement with error bounds (dgerfs_), condition estimate (dgecon_),
equilibration (dgeequ_/dlaqge_) and the expert driver (dgesvx_) on the GPU,
against the reference's own results (tests/golden, from the compiled FLENS
shims; inputs with one badly scaled row and column).

Bars:
* geequ / laqge are exact operations: bitwise equal to the reference;
* refined solutions within 1e-12 normwise of the reference's; berr, the
  componentwise backward error, <= n eps for both;
* rcond (an estimate from GPU solves and parallel sums) within a relative
  1e-6 of the reference's; ferr within a factor of 2 of the reference's:
  ferr = || |inv(A)| (|r| + nz eps (|A||x| + |b|)) || / ||x|| where the final
  residual r is roundoff noise bounded by the eps term (the GPU forms it
  with fused multiply-adds: at n = 1 its exact residual is nonzero where
  the reference's rounded one is 0), so each estimate lies between the eps
  term's norm and twice it;
* dgesvx: same INFO, reciprocal pivot growth, EQUED reporting the scaling
  actually applied (the reference's shim returns 'N' there).
"""
import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def within_2x(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return bool(((a <= 2 * b) & (b <= 2 * a) & (a > 0)).all())


def test_gecon_gerfs_vs_reference(golden, port):
    for i, (name, n) in enumerate(G.refine_case_list()):
        A, Ae, B = G.refine_inputs(i, n)
        LU = A.copy(order="F")
        piv, _ = port.dgetrf(LU)
        rc = []
        for nm in ("1", "I"):
            r, info = fg.dgecon(nm, LU.copy(order="F"), port.dlange(nm, A))
            assert info == 0
            rc.append(r)
        assert rel(rc, golden[name + "_rcond"]) <= 1e-6, (name, rc)
        for tr in "NT":
            X = B.copy(order="F")
            port.dgetrs(tr, LU, piv, X)
            X[0, :] += 1e-8
            ferr, berr, info = fg.dgerfs(tr, A, LU.copy(order="F"), piv, B, X)
            assert info == 0
            assert oracle.normwise_rel(X, golden[name + f"_rfs{tr}_X"]) <= 1e-12, (name, tr)
            assert (berr <= n * EPS).all() and (golden[name + f"_rfs{tr}_berr"] <= n * EPS).all()
            assert within_2x(ferr, golden[name + f"_rfs{tr}_ferr"]), (name, tr, ferr)


def test_geequ_laqge_bitwise(golden, port):
    for i, (name, n) in enumerate(G.refine_case_list()):
        A, Ae, B = G.refine_inputs(i, n)
        r, c, rcnd, ccnd, amax, info = fg.dgeequ(Ae.copy(order="F"))
        assert np.array_equal(np.concatenate([r, c, [rcnd, ccnd, amax, info]]), golden[name + "_equ"])
        a1, a2 = Ae.copy(order="F"), Ae.copy(order="F")
        assert fg.dlaqge(a1, r, c, rcnd, ccnd, amax) == port.dlaqge(a2, r, c, rcnd, ccnd, amax)
        assert np.array_equal(a1, a2)


def test_gesvx_vs_reference(golden):
    for i, (name, n) in enumerate(G.refine_case_list()):
        A, Ae, B = G.refine_inputs(i, n)
        for fact in "NE":
            for tr in "NT":
                Aw, Bw = Ae.copy(order="F"), B.copy(order="F")
                AF, X = np.zeros((n, n), order="F"), np.zeros((n, 3), order="F")
                pv = np.zeros(n, dtype=np.int32)
                info, eq, rcn, fe, be, g = fg.dgesvx(fact, tr, Aw, AF, pv, "N", np.zeros(n),
                                                     np.zeros(n), Bw, X)
                k = name + f"_svx{fact}{tr}"
                ref = golden[k + "_s"]
                assert info == int(ref[0]), k
                assert rel([rcn, g], ref[1:3]) <= 1e-6, (k, rcn, g)
                assert oracle.normwise_rel(X, golden[k + "_X"]) <= 1e-12, k
                assert np.array_equal(Aw, golden[k + "_A"]), k            # equilibrated A
                assert oracle.normwise_rel(AF, golden[k + "_AF"]) <= 1e-12, k
                assert within_2x(fe, ref[3:3 + 3]), (k, fe, ref[3:3 + 3])
                assert (be <= n * EPS).all(), k
                assert (eq == "N") == np.array_equal(Aw, Ae), k
    # singular: INFO, pivot growth, rcond 0, X untouched
    A = G.singular_input()
    n = A.shape[0]
    AF, X = np.zeros((n, n), order="F"), np.full((n, 1), 7.0, order="F")
    info, eq, rcn, fe, be, g = fg.dgesvx("N", "N", A, AF, np.zeros(n, dtype=np.int32), "N",
                                         np.zeros(n), np.zeros(n), G.U(7778, n, 1), X)
    ref = golden["svx_sing_s"]
    assert info == int(ref[0]) == 3 and rcn == 0.0
    assert rel([g], [ref[2]]) <= 1e-12
    assert (X == 7.0).all()


def test_gesvx_factored_and_large(cuda, port):
    """FACT = 'F' reuses given factors; a larger well-conditioned system
    through the device entry point."""
    import ctypes
    import torch
    n = 600
    A = oracle.uniform(np.random.default_rng(3), n, n)
    A[np.arange(n), np.arange(n)] += n / 4
    B = oracle.uniform(np.random.default_rng(4), n, 2)
    LU = A.copy(order="F")
    piv, _ = port.dgetrf(LU)
    X = np.zeros((n, 2), order="F")
    info, eq, rcn, fe, be, g = fg.dgesvx("F", "N", A.copy(order="F"), LU.copy(order="F"), piv.copy(),
                                         "N", np.zeros(n), np.zeros(n), B.copy(order="F"), X)
    assert info == 0 and eq == "N"
    Xr = B.copy(order="F")
    port.dgesv(A.copy(order="F"), Xr)
    assert oracle.normwise_rel(X, Xr) <= 1e-12
    assert (be <= n * EPS).all() and (fe < 1e-10).all()
    dev = lambda M: fg.to_colmajor(torch.from_numpy(M).to(cuda))
    dA, dAF, dB, dX = dev(A), dev(np.zeros((n, n))), dev(B), dev(np.zeros((n, 2)))
    dp = torch.zeros(n, dtype=torch.int32, device=cuda)
    dr, dc = torch.zeros(n, dtype=torch.float64, device=cuda), torch.zeros(n, dtype=torch.float64, device=cuda)
    eqb = ctypes.create_string_buffer(b"N", 2)
    rc, rp = ctypes.c_double(), ctypes.c_double()
    fe2, be2 = np.zeros(2), np.zeros(2)
    inf = ctypes.c_int()
    st = fg.lib().flens_gb300_dgesvx(b"E", b"N", n, 2, dA.data_ptr(), n, dAF.data_ptr(), n, dp.data_ptr(),
                                     eqb, dr.data_ptr(), dc.data_ptr(), dB.data_ptr(), n, dX.data_ptr(), n,
                                     ctypes.byref(rc), fe2.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     be2.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(rp),
                                     ctypes.byref(inf), None)
    assert st == 0 and inf.value == 0
    assert oracle.normwise_rel(dX.cpu().numpy(), Xr) <= 1e-12
    assert rel([rc.value], [rcn]) <= 1e-6
