"""dtrmm_, dsymm_, dsyr2k_ on the GPU against the reference's own results
(tests/golden, from the compiled FLENS shims) and, at larger sizes, against
the oracle (restated cxxblas trmm/symm/syr2k, bitwise equal to the reference).

Bar: normwise relative error <= 1e-13, the same as for gemm (the products run
on the FP64 GEMM engine with a different summation order); syr2k leaves the
other triangle of C untouched.
"""
import numpy as np
import pytest

import flens_gb300 as fg
import make_golden as G
import oracle

pytestmark = pytest.mark.gpu


def test_trmm_vs_reference(golden):
    for i, (name, (m, n, side, uplo, ta, diag, alpha)) in enumerate(G.trmm_case_list()):
        A, B = G.trmm_inputs(i, m, n, side)
        out = fg.dtrmm(side, uplo, ta, diag, alpha, A, B.copy(order="F"))
        if m == 0 or n == 0:
            assert np.array_equal(out, golden[name]), name
            continue
        assert oracle.normwise_rel(out, golden[name]) <= 1e-13, name


def test_symm_vs_reference(golden):
    for i, (name, (m, n, side, uplo, a, b)) in enumerate(G.symm_case_list()):
        A, B, C = G.symm_inputs(i, m, n, side)
        out = fg.dsymm(side, uplo, a, A, B, b, C.copy(order="F"))
        if m == 0 or n == 0:
            continue
        assert oracle.normwise_rel(out, golden[name]) <= 1e-13, name


def test_syr2k_vs_reference(golden):
    for i, (name, (n, k, uplo, tr, a, b)) in enumerate(G.syr2k_case_list()):
        A, B, C0 = G.syr2k_inputs(i, n, k, tr)
        out = fg.dsyr2k(uplo, tr, a, A, B, b, C0.copy(order="F"))
        if n == 0:
            continue
        mask = np.tril(np.ones((n, n))) if uplo == "L" else np.triu(np.ones((n, n)))
        assert np.array_equal(out[mask == 0], C0[mask == 0]), name
        assert oracle.normwise_rel(out * mask, golden[name] * mask) <= 1e-13, name


@pytest.mark.parametrize("side", ["L", "R"])
def test_device_level3_large(cuda, port, side):
    import torch
    rng = np.random.default_rng(11)
    m, n = 700, 900
    ka = m if side == "L" else n
    dev = lambda X: fg.to_colmajor(torch.from_numpy(X).to(cuda))
    for uplo in "LU":
        A = oracle.uniform(rng, ka, ka)
        B = oracle.uniform(rng, m, n)
        for ta in "NT":
            for diag in "NU":
                Bd = dev(B)
                lib_st = fg.lib().flens_gb300_dtrmm(side.encode(), uplo.encode(), ta.encode(),
                                                    diag.encode(), m, n, -0.5, dev(A).data_ptr(),
                                                    ka, Bd.data_ptr(), m, None)
                assert lib_st == 0
                want = port.dtrmm(side, uplo, ta, diag, -0.5, A, B.copy(order="F"))
                assert oracle.normwise_rel(Bd.cpu().numpy(), want) <= 1e-13
        C = oracle.uniform(rng, m, n)
        Cd = dev(C)
        assert fg.lib().flens_gb300_dsymm(side.encode(), uplo.encode(), m, n, 1.5, dev(A).data_ptr(),
                                          ka, dev(B).data_ptr(), m, 0.5, Cd.data_ptr(), m, None) == 0
        want = port.dsymm(side, uplo, 1.5, A, B, 0.5, C.copy(order="F"))
        assert oracle.normwise_rel(Cd.cpu().numpy(), want) <= 1e-13
