"""CPU checks of the split-precision GEMM algorithm (the NumPy model that the
GPU code is compared with bit for bit): the group plan covers every slice
pair of the truncated triangle once per k range and keeps every tensor-core
sum exact, and the algorithm is as accurate as the reference's FP64 gemm
(cxxblas/level3/gemm.tcc:42-190, through the oracle port)."""
import numpy as np
import pytest

import oracle
import split_model as sm

EPS = np.finfo(np.float64).eps


def wide_range(seed, m, n, E):
    rng = np.random.default_rng(seed)
    return np.ldexp(rng.uniform(-1.0, 1.0, (m, n)), rng.integers(-E, E + 1, (m, n)))


@pytest.mark.parametrize("bits", [4, 5, 6, 7, 8])
@pytest.mark.parametrize("S", [1, 2, 5, 9, 13])
@pytest.mark.parametrize("K", [1, 64, 100, 4096, 4097, 8192, 20000])
def test_plan_covers_triangle_exactly(bits, S, K):
    P = 1 << (2 * (bits - 1))
    Kp = sm.kpad(K)
    cover = {}
    for (dg, slo, shi, k0, k1) in sm.plan_groups(bits, S, K):
        assert 2 <= dg <= S + 1 and 1 <= slo <= shi <= dg - 1
        assert 0 <= k0 < k1 <= Kp and (k1 - k0) % sm.BK == 0
        assert (shi - slo + 1) * (k1 - k0) * P <= sm.ACC_LIMIT
        if shi > slo:
            assert (k0, k1) == (0, Kp)           # multi-pair runs span the whole K
        for s in range(slo, shi + 1):
            for k in range(k0, k1, sm.BK):
                key = (s, dg - s, k)
                assert key not in cover
                cover[key] = True
    want = {(s, t, k) for s in range(1, S + 1) for t in range(1, S + 1) if s + t <= S + 1
            for k in range(0, Kp, sm.BK)}
    assert set(cover) == want


def test_digits_reconstruct_and_are_bounded():
    X = wide_range(3, 20, 300, 30)
    X[4, :] = 0.0
    e, _, _ = sm.row_exponents(X)
    for bits in (5, 7, 8):
        S = 12
        d = sm.digits(X, e, bits, S)
        assert np.abs(d).max() <= 1 << (bits - 1)
        rec = sum(np.ldexp(d[s].astype(np.float64), (e - bits * (s + 1))[:, None].astype(np.int32))
                  for s in range(S))
        err = np.abs(rec - X)
        assert (err <= np.ldexp(1.0, (e - bits * S - 1).astype(np.int32))[:, None] * 1.0001).all()


def test_digits_equal_rounded_prefixes():
    # d_s = R_s - 2^beta R_{s-1}, R_s = rint(x 2^(beta (s-1))) (half to even):
    # the integer form the GPU evaluates; exact rational arithmetic here
    from fractions import Fraction
    bits, S = 7, 9
    vals = [0.5, 1.5, 2.5, -0.5, -2.5, 63.5, -63.5]
    vals += [3 + 0.5 * 2.0 ** (-bits * l) for l in range(1, 7)]
    vals += [-(1 + 0.5 * 2.0 ** (-bits * l)) for l in range(1, 7)]
    vals += list(np.random.default_rng(3).uniform(-63.9, 63.9, 200))
    X = np.ldexp(np.array(vals)[:, None], 8 - bits)           # row exponent e = 8
    d = sm.digits(X, np.full(len(vals), 8), bits, S)[:, :, 0]

    def rint(q):
        f = q.numerator // q.denominator
        r = q - f
        return f + 1 if r > Fraction(1, 2) or (r == Fraction(1, 2) and f % 2) else f

    for i, x in enumerate(vals):
        prev = 0
        for s in range(S):
            R = rint(Fraction(x) * 2 ** (bits * s))
            assert d[s, i] == R - (prev << bits), (x, s)
            prev = R


@pytest.mark.parametrize("E,want_slices", [(0, 8), (16, 9), (48, 9)])
def test_model_accuracy(port, E, want_slices):
    m, n, k = 40, 48, 1024
    A = wide_range(10 + E, m, k, E)
    B = wide_range(20 + E, k, n, E)
    S = sm.slices_for(A, B, 7)
    assert S == want_slices
    C = sm.split_gemm_model(1.0, A, B, 0.0, np.zeros((m, n)), 7, S)
    exact = sm.exact_gemm(A, B)
    Cref = np.zeros((m, n), order="F")
    port.dgemm("N", "N", 1.0, np.asfortranarray(A), np.asfortranarray(B), 0.0, Cref)
    assert oracle.normwise_rel(C, Cref) <= 1e-13
    # elementwise no worse than the reference's sequential FP64 loop, and
    # componentwise well inside FP64's a-priori bound K*u*|A||B|
    rel = lambda X: (np.abs(X - exact) / np.abs(exact)).max()
    assert rel(C) <= max(rel(Cref), 8 * EPS)
    assert (np.abs(C - exact) / (np.abs(A) @ np.abs(B))).max() <= 64 * EPS


def test_model_beta_and_alpha():
    A = wide_range(1, 10, 70, 3)
    B = wide_range(2, 70, 12, 3)
    C0 = wide_range(3, 10, 12, 0)
    C = sm.split_gemm_model(-2.5, A, B, 0.5, C0.copy(), 7, 9)
    np.testing.assert_allclose(C, 0.5 * C0 - 2.5 * sm.exact_gemm(A, B), rtol=0, atol=1e-13)
