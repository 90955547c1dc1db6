"""NumPy model of the split-precision FP64 GEMM (flens_gb300_dgemm_split).

The model performs the same arithmetic as the GPU code, step for step, so a
GPU result can be compared with it bit for bit:

* every row i of op(A) gets an exponent e_i (amax_i < 2^(e_i - 1)) and is
  written as balanced base-2^beta digits a_ik = 2^e_i * sum_s d_s 2^(-beta s),
  |d_s| <= 2^(beta-1), by repeated rint / subtract / scale, which is exact in
  FP64; columns j of op(B) likewise with exponents f_j;
* the digit products of slice pairs (s, t) with s + t = dg <= S + 1 are
  summed over k in FP32 on the tensor cores; every group of pairs and k range
  is small enough that all partial sums are integers of magnitude <= 2^24, so
  the sums are exact (here: int64 matmul);
* the group sums of one diagonal dg share the scale 2^(e_i + f_j - beta*dg):
  they are added exactly as integers, in segments of at most SEG_GROUPS
  groups (in the diagonal's group order), and each segment's integer sum,
  scaled exactly, is added in FP64, largest dg first, S = S + I * 2^(...)
  (one rounding per segment); C = (beta*C) + (alpha*S) at the end.

The digits are the balanced base-2^beta digits of x = a 2^(beta - e_i),
d_s = R_s - 2^beta R_{s-1} with R_s = rint(x 2^(beta (s-1))) (round half to
even); repeated rint / subtract / scale in FP64 gives the same digits, because
2^beta R_{s-1} is an even integer.

`exact_gemm` gives the correctly rounded product for judging accuracy.
"""
import math

import numpy as np

ACC_LIMIT = 1 << 24          # exact FP32 integer range
SEG_GROUPS = 127             # groups per exact int32 segment sum: 127 * 2^24 < 2^31
BK = 64                      # k-block of the tensor-core kernel (bf16: 128 bytes)


def row_exponents(X):
    """e_i with amax_i < 2^(e_i - 1) (0 for a zero row), nnz and sum|x| per row."""
    ax = np.abs(X)
    amax = ax.max(axis=1) if X.shape[1] else np.zeros(X.shape[0])
    _, ex = np.frexp(amax)                   # amax = m 2^ex, m in [0.5, 1)
    e = np.where(amax > 0, ex + 1, 0).astype(np.int64)
    return e, np.count_nonzero(X, axis=1), ax.sum(axis=1)


def digits(X, e, beta, S):
    """Balanced digits, shape (S, rows, K), int64; X = 2^e * sum d_s 2^(-beta s)
    up to a remainder below 2^(e - beta S - 1)."""
    x = np.ldexp(X, (beta - e)[:, None].astype(np.int32))
    out = np.empty((S,) + X.shape, dtype=np.int64)
    for s in range(S):
        d = np.rint(x)
        out[s] = d.astype(np.int64)
        x = (x - d) * float(1 << beta)
    return out


def kpad(K):
    return (K + BK - 1) // BK * BK


def plan_groups(beta, S, K):
    """Groups (dg, s_lo, s_hi, k0, k1) in summation order: dg from S+1 down to
    2, pairs (s, dg - s) for s in [s_lo, s_hi] (1-based slices), k in [k0, k1).
    Each group keeps (#pairs) * (k1 - k0) * 4^(beta-1) <= 2^24.  When K has to
    be cut into chunks a group holds one pair; otherwise `per` pairs over the
    whole padded K (consecutive slices, contiguous in the concatenated
    layout)."""
    P = 1 << (2 * (beta - 1))
    Kp = kpad(K)
    kc = min(Kp, (ACC_LIMIT // P) // BK * BK)
    if kc <= 0:
        raise ValueError("slice width too large for exact accumulation")
    nchunks = (Kp + kc - 1) // kc
    per = ACC_LIMIT // (P * Kp) if nchunks == 1 else 1
    groups = []
    for dg in range(S + 1, 1, -1):
        if nchunks == 1:
            s = 1
            while s <= dg - 1:
                hi = min(dg - 1, s + per - 1)
                groups.append((dg, s, hi, 0, Kp))
                s = hi + 1
        else:
            for c in range(nchunks):
                for s in range(1, dg):
                    groups.append((dg, s, s, c * kc, min(Kp, (c + 1) * kc)))
    return groups


def split_gemm_model(alpha, opA, opB, beta_c, C, beta, S):
    """C <- beta_c*C + alpha*opA@opB the way the GPU computes it (C modified
    and returned).  opA: M x K, opB: K x N (float64)."""
    M, K = opA.shape
    N = opB.shape[1]
    e, _, _ = row_exponents(opA)
    f, _, _ = row_exponents(opB.T)
    # digit products as float64 matmuls: integers below 2^53, so exact in any order
    dA = digits(opA, e, beta, S).astype(np.float64)
    dB = digits(opB.T, f, beta, S).astype(np.float64)
    Ssum = np.zeros((M, N))
    groups = plan_groups(beta, S, K)
    seg = None            # exact integer sum of the open segment
    gi = 0                # index of the group within its diagonal
    for idx, (dg, slo, shi, k0, k1) in enumerate(groups):
        if idx > 0 and groups[idx - 1][0] != dg:
            gi = 0
        k1 = min(k1, K)
        if k0 >= k1:
            acc = np.zeros((M, N))
        else:
            acc = sum(dA[s - 1][:, k0:k1] @ dB[dg - s - 1][:, k0:k1].T for s in range(slo, shi + 1))
        assert np.abs(acc).max(initial=0) <= ACC_LIMIT
        seg = acc if gi % SEG_GROUPS == 0 else seg + acc
        assert np.abs(seg).max(initial=0) < 2 ** 31
        last_of_diag = idx == len(groups) - 1 or groups[idx + 1][0] != dg
        if gi % SEG_GROUPS == SEG_GROUPS - 1 or last_of_diag:
            Ssum += np.ldexp(seg, (e[:, None] + f[None, :] - beta * dg).astype(np.int32))
        gi += 1
    C[...] = (beta_c * C) + (alpha * Ssum)
    return C


def exact_gemm(A, B):
    """Correctly rounded A @ B (float64): exact products by Veltkamp/Dekker
    splitting, exact sums by math.fsum.  For small sizes only."""
    M, K = A.shape
    N = B.shape[1]
    split = 134217729.0                              # 2^27 + 1

    def veltkamp(x):
        c = split * x
        hi = c - (c - x)
        return hi, x - hi

    ah, al = veltkamp(A)
    bh, bl = veltkamp(B)
    out = np.empty((M, N))
    for j in range(N):
        p = A * B[:, j][None, :]
        # error of the rounded product: exact by Dekker's two-product
        e = ((ah * bh[:, j] - p) + ah * bl[:, j] + al * bh[:, j]) + al * bl[:, j]
        for i in range(M):
            out[i, j] = math.fsum(np.concatenate([p[i], e[i]]))
    return out


def slices_for(opA, opB, beta, target_bits=51):
    """Slice count the library chooses: beta*S >= target_bits + 2 + log2 of the
    worst ratio (2^e_i * nnz_i / sum_k |a_ik|) over rows of op(A) and columns of
    op(B), which bounds how much the digit truncation error exceeds u*|A||B|."""
    worst = 1.0
    for X in (opA, opB.T):
        e, nnz, s = row_exponents(X)
        ok = s > 0
        if ok.any():
            r = np.ldexp(nnz[ok].astype(np.float64), e[ok].astype(np.int32)) / s[ok]
            worst = max(worst, float(r.max()))
    m, ex = math.frexp(worst)                        # worst = m 2^ex, m in [0.5, 1)
    bits = target_bits + 2 + (ex - 1 if m == 0.5 else ex)
    return min(20, -(-bits // beta))
