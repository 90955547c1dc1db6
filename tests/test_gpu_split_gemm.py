"""Split-precision FP64 GEMM (flens_gb300_dgemm_split) on the GPU.

Three bars:
* bit-for-bit equality with the NumPy model of the algorithm (split_model),
  which holds only if every tensor-core sum of digit products is exact;
* the reference's own gemm (the oracle port of cxxblas::gemm,
  cxxblas/level3/gemm.tcc:42-190) to the plain-gemm tolerance, normwise
  <= 1e-13;
* against the correctly rounded product: elementwise relative error no worse
  than the sequential FP64 loop's and componentwise error <= 64 u (|A||B|)_ij
  (FP64's own a-priori bound is K u |A||B|), on inputs u*2^e with u
  uniform[-1,1] and e uniform in [-E, E] for E in {0, 16, 48}.
"""
import numpy as np
import pytest

import flens_gb300 as fg
import oracle
import split_model as sm

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps
BITS = 7


def wide_range(seed, m, n, E):
    rng = np.random.default_rng(seed)
    return np.ldexp(rng.uniform(-1.0, 1.0, (m, n)), rng.integers(-E, E + 1, (m, n)))


def dev(cuda, X):
    import torch
    return fg.to_colmajor(torch.from_numpy(np.asfortranarray(X)).to(cuda))


def op(X, t):
    return X if t == "N" else X.T


def run_split(cuda, ta, tb, alpha, A, B, beta, C, slices=0):
    dA, dB, dC = dev(cuda, A), dev(cuda, B), dev(cuda, C)
    used = fg.dgemm_split_dev(ta, tb, alpha, dA, dB, beta, dC, slices=slices)
    return dC.cpu().numpy(), used


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("E", [0, 16, 48])
def test_split_bitwise_vs_model(cuda, ta, tb, E):
    m, n, k = 150, 290, 333
    A = wide_range(11 + E, *((m, k) if ta == "N" else (k, m)), E)
    B = wide_range(12 + E, *((k, n) if tb == "N" else (n, k)), E)
    C = wide_range(13, m, n, 0)
    alpha, beta = 1.5, 0.5
    got, used = run_split(cuda, ta, tb, alpha, A, B, beta, C)
    assert used == sm.slices_for(op(A, ta), op(B, tb), BITS)
    want = sm.split_gemm_model(alpha, op(A, ta), op(B, tb), beta, C.copy(), BITS, used)
    np.testing.assert_array_equal(got, want)


def test_split_exact_at_accumulator_limit(cuda):
    # first digits all in [50, 64] and one K chunk of 4096: the digit-product
    # sums of that chunk fill all 24 bits of the FP32 accumulator
    rng = np.random.default_rng(5)
    m, n, k = 128, 256, 4096
    A = rng.uniform(100.0, 127.0, (m, k))
    B = rng.uniform(100.0, 127.0, (k, n))
    C = np.zeros((m, n))
    got, used = run_split(cuda, "N", "N", 1.0, A, B, 0.0, C, slices=3)
    assert used == 3
    e, _, _ = sm.row_exponents(A)
    d1 = sm.digits(A, e, BITS, 1)[0]
    assert np.abs(d1).min() >= 50
    want = sm.split_gemm_model(1.0, A, B, 0.0, C.copy(), BITS, 3)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("E,slices", [(0, 8), (16, 9), (48, 9)])
def test_split_accuracy(cuda, port, E, slices):
    m, n, k = 96, 112, 2048
    A = wide_range(100 + E, m, k, E)
    B = wide_range(200 + E, k, n, E)
    C = np.zeros((m, n))
    got, used = run_split(cuda, "N", "N", 1.0, A, B, 0.0, C)
    assert used == slices
    # the reference's gemm (sequential FP64) on the same inputs
    Cref = np.zeros((m, n), order="F")
    port.dgemm("N", "N", 1.0, np.asfortranarray(A), np.asfortranarray(B), 0.0, Cref)
    assert oracle.normwise_rel(got, Cref) <= 1e-13
    exact = sm.exact_gemm(A, B)
    cw = np.abs(got - exact) / (np.abs(A) @ np.abs(B))
    assert cw.max() <= 64 * EPS, cw.max()
    # no worse than the sequential FP64 loop, elementwise
    rel = np.abs(got - exact) / np.abs(exact)
    rel_ref = np.abs(Cref - exact) / np.abs(exact)
    assert rel.max() <= max(rel_ref.max(), 8 * EPS)


def test_split_alpha_beta_and_quick_returns(cuda):
    import torch
    A = wide_range(1, 40, 30, 4)
    B = wide_range(2, 30, 50, 4)
    C = wide_range(3, 40, 50, 0)
    # k == 0 and alpha == 0: C = beta*C only (multiply, as cxxblas gescal)
    got, used = run_split(cuda, "N", "N", 2.0, A[:, :0], B[:0, :], 0.25, C)
    np.testing.assert_array_equal(got, C * 0.25)
    assert used == 0
    got, used = run_split(cuda, "N", "N", 0.0, A, B, -3.0, C)
    np.testing.assert_array_equal(got, C * -3.0)
    # m == 0 / n == 0 are no-ops
    dC = dev(cuda, C)
    fg.dgemm_split_dev("N", "N", 1.0, dev(cuda, A[:0, :]), dev(cuda, B), 1.0, dC[:0, :])
    fg.dgemm_split_dev("N", "N", 1.0, dev(cuda, A), dev(cuda, B[:, :0]), 1.0, dC[:, :0])
    np.testing.assert_array_equal(dC.cpu().numpy(), C)
    # negative alpha, beta != 0, fixed slice count: still the model, bit for bit
    got, used = run_split(cuda, "T", "N", -0.75, A.T.copy(), B, 2.0, C, slices=4)
    assert used == 4
    want = sm.split_gemm_model(-0.75, A, B, 2.0, C.copy(), BITS, 4)
    np.testing.assert_array_equal(got, want)
    torch.cuda.synchronize()


def test_split_zero_rows_and_columns(cuda):
    A = wide_range(7, 70, 90, 8)
    B = wide_range(8, 90, 60, 8)
    A[5, :] = 0.0
    A[:, 17] = 0.0
    B[:, 9] = 0.0
    C = np.zeros((70, 60))
    got, used = run_split(cuda, "N", "N", 1.0, A, B, 0.0, C)
    want = sm.split_gemm_model(1.0, A, B, 0.0, C.copy(), BITS, used)
    np.testing.assert_array_equal(got, want)
    assert not got[5, :].any() and not got[:, 9].any()


@pytest.mark.parametrize("case", ["inf", "nan", "huge", "tiny"])
def test_split_falls_back_to_fp64_kernel(cuda, case):
    A = wide_range(9, 33, 44, 2)
    B = wide_range(10, 44, 55, 2)
    if case == "inf":
        A[3, 7] = np.inf
    elif case == "nan":
        B[4, 2] = np.nan
    elif case == "huge":
        A *= 2.0 ** 600
        B *= 2.0 ** 500
    else:
        A *= 2.0 ** -600
        B *= 2.0 ** -400
    C = wide_range(11, 33, 55, 0)
    got, used = run_split(cuda, "N", "N", 1.0, A, B, 0.5, C)
    assert used == -1
    dC = dev(cuda, C)
    fg.dgemm_dev("N", "N", 1.0, dev(cuda, A), dev(cuda, B), 0.5, dC)
    np.testing.assert_array_equal(got, dC.cpu().numpy())


def test_split_argument_errors(cuda):
    import ctypes
    L = fg.lib()
    used = ctypes.c_int(0)
    f = L.flens_gb300_dgemm_split
    ok = dict(ta=b"N", tb=b"N", m=4, n=4, k=4, lda=4, ldb=4, ldc=4, s=0)

    def call(**kw):
        a = dict(ok, **kw)
        return f(a["ta"], a["tb"], a["m"], a["n"], a["k"], 1.0, None, a["lda"], None, a["ldb"], 0.0,
                 None, a["ldc"], a["s"], ctypes.byref(used), None)

    assert call(ta=b"X") == -1
    assert call(tb=b"?") == -2
    assert call(m=-1) == -3
    assert call(n=-1) == -4
    assert call(k=-1) == -5
    assert call(lda=3) == -8
    assert call(ldb=3) == -10
    assert call(ldc=3) == -13
    assert call(s=-1) == -14
    assert call(s=21) == -14


@pytest.mark.slow
def test_split_full_size_wide_range(cuda, port):
    """M = N = K = 8192, E = 48: 9 slices; a 64-row sample against the oracle
    and the whole product against the GPU's plain FP64 gemm."""
    import torch
    n = 8192
    g = torch.Generator(device=cuda).manual_seed(48)

    def gen():
        u = torch.rand(n, n, generator=g, device=cuda, dtype=torch.float64) * 2 - 1
        e = torch.randint(-48, 49, (n, n), generator=g, device=cuda)
        return torch.ldexp(u, e.to(torch.float64)).t().contiguous().t()

    A, B = gen(), gen()
    C = torch.zeros((n, n), dtype=torch.float64, device=cuda).t()
    used = fg.dgemm_split_dev("N", "N", 1.0, A, B, 0.0, C)
    assert used == 9
    C64 = torch.zeros((n, n), dtype=torch.float64, device=cuda).t()
    fg.dgemm_dev("N", "N", 1.0, A, B, 0.0, C64)
    assert oracle.normwise_rel(C.cpu().numpy(), C64.cpu().numpy()) <= 1e-13
    rows = np.sort(np.random.default_rng(0).choice(n, 64, replace=False))
    As = np.asfortranarray(A.cpu().numpy()[rows, :])
    Bh = np.asfortranarray(B.cpu().numpy())
    Cs = np.zeros((64, n), order="F")
    port.dgemm("N", "N", 1.0, As, Bh, 0.0, Cs)
    assert oracle.normwise_rel(C.cpu().numpy()[rows, :], Cs) <= 1e-13


def test_split_bitwise_vs_model_several_groups_per_diagonal(cuda):
    # k = 2048: one K chunk, one slice pair per group, so every diagonal dg
    # has dg - 1 groups whose exact integer sums are added before the FP64 sum
    m, n, k = 130, 270, 2048
    A = wide_range(31, m, k, 16)
    B = wide_range(32, k, n, 16)
    C = wide_range(33, m, n, 0)
    got, used = run_split(cuda, "N", "N", 1.5, A, B, 0.5, C)
    want = sm.split_gemm_model(1.5, A, B, 0.5, C.copy(), BITS, used)
    np.testing.assert_array_equal(got, want)
