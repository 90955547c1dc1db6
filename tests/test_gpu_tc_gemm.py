"""tcgen05 low-precision GEMM (flens_gb300_sgemm_tc) against an FP64 torch
reference of the same op on the same rounded operands (the torch FP64
reference of the same op that numerics tests of a CUDA kernel use).

The kernel rounds op(A) and op(B) to TF32 (round to nearest, ties away),
BF16 (round to nearest even) or FP8 e4m3 (per-row / per-column scale
amax/448, round to nearest even) and accumulates in FP32 on the tensor cores.
The reference applies the same rounding in torch and multiplies in FP64, so
the only difference left is FP32 accumulation order: the bar is a normwise
relative error <= 1e-5 and an elementwise error <= 1e-4 * (|alpha||A||B| +
|beta||C|).
"""
import ctypes

import numpy as np
import pytest

import flens_gb300 as fg

pytestmark = pytest.mark.gpu

PREC = {"tf32": 0, "bf16": 1, "fp8": 2, "fp8x2": 5, "fp8x3": 6}


def round_tf32(x):
    import torch
    b = x.contiguous().view(torch.int32)
    r = ((b + 0x1000) & ~0x1FFF)          # round half away from zero on the magnitude
    return r.view(torch.float32)


def round_op(x, prec, rows_dim):
    """x: fp32 tensor holding op(X) as (rows, K); returns the dequantised fp64 operand."""
    import torch
    if prec == "bf16":
        return x.to(torch.bfloat16).to(torch.float64)
    if prec == "tf32":
        return round_tf32(x).to(torch.float64)
    amax = x.abs().amax(dim=1, keepdim=True)
    s = torch.where(amax > 0, amax / 448.0, torch.ones_like(amax))
    q = (x * (1.0 / s)).to(torch.float8_e4m3fn)
    return q.to(torch.float64) * s.to(torch.float64)


def sgemm_tc(prec, ta, tb, alpha, A, B, beta, C):
    import torch
    m, n = C.shape
    k = A.shape[1] if ta == "N" else A.shape[0]
    L = fg.lib()
    f = L.flens_gb300_sgemm_tc
    f.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_int
    st = f(PREC[prec], ta.encode(), tb.encode(), m, n, k, alpha, A.data_ptr(), A.stride(1),
           B.data_ptr(), B.stride(1), beta, C.data_ptr(), C.stride(1),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, fg.last_error()
    torch.cuda.synchronize()
    L2 = fg.lib().flens_gb300_sync(None)
    assert L2 == 0, fg.last_error()
    return C


def colmajor(torch, rows, cols, seed, dev):
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    return torch.rand((cols, rows), generator=g, dtype=torch.float32, device=dev).mul_(2).sub_(1).t()


@pytest.mark.parametrize("prec", ["bf16", "tf32", "fp8"])
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (200, 300, 100), (1000, 600, 256),
                                   (257, 513, 1000), (64, 40, 512)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T")])
def test_sgemm_tc_vs_fp64_reference(cuda, prec, m, n, k, ta, tb):
    import torch
    A = colmajor(torch, m if ta == "N" else k, k if ta == "N" else m, 1 + m, cuda)
    B = colmajor(torch, k if tb == "N" else n, n if tb == "N" else k, 2 + n, cuda)
    C0 = colmajor(torch, m, n, 3 + k, cuda)
    alpha, beta = -1.0, 1.0
    opA = A if ta == "N" else A.t()                 # (m, k)
    opB = B if tb == "N" else B.t()                 # (k, n)
    Ar = round_op(opA, prec, 0)                     # rows of op(A) scaled
    Br = round_op(opB.t(), prec, 0).t()             # columns of op(B) scaled
    ref = alpha * (Ar @ Br) + beta * C0.to(torch.float64)
    bound = abs(alpha) * (Ar.abs() @ Br.abs()) + abs(beta) * C0.abs().to(torch.float64)
    C = C0.clone()
    sgemm_tc(prec, ta, tb, alpha, A, B, beta, C)
    err = (C.to(torch.float64) - ref)
    rel = (err.norm() / ref.norm()).item()
    elem = (err.abs() / bound.clamp_min(1e-30)).max().item()
    # FP8 (kind::f8f6f4) products are summed with less than FP32 precision
    # inside the tensor core: at K <= 256 (the LU trailing-update depth) the
    # FP32 bar holds; over K ~ 1000 the measured error is ~2e-4, so the bar
    # there is 1e-3.
    tol_rel, tol_elem = (1e-5, 1e-4) if (prec != "fp8" or k <= 256) else (1e-3, 1e-3)
    assert rel <= tol_rel and elem <= tol_elem, (rel, elem)


def test_sgemm_tc_beta_semantics(cuda):
    # beta scales C by a multiply, as the reference's gescal does: a NaN in C
    # survives beta == 0; alpha == 0 leaves beta*C and reads neither A nor B
    import torch
    m, n, k = 300, 260, 128
    A = colmajor(torch, m, k, 7, cuda)
    B = colmajor(torch, k, n, 8, cuda)
    C = colmajor(torch, m, n, 9, cuda).clone()
    C[5, 7] = float("nan")
    sgemm_tc("bf16", "N", "N", 2.5, A, B, 0.0, C)
    ref = 2.5 * (A.to(torch.bfloat16).double() @ B.to(torch.bfloat16).double())
    assert torch.isnan(C[5, 7])
    mask = torch.ones_like(ref, dtype=torch.bool)
    mask[5, 7] = False
    assert ((C.double() - ref)[mask].norm() / ref[mask].norm()).item() <= 1e-5
    C2 = colmajor(torch, m, n, 10, cuda).clone()
    C20 = C2.clone()
    An = torch.full_like(A, float("nan"))
    sgemm_tc("bf16", "N", "N", 0.0, An, B, 0.5, C2)
    assert torch.equal(C2, 0.5 * C20)


def fp8_terms(x, nterms):
    """Per-row scale amax/448 and the e4m3 terms of the scaled rows of x
    (fp32, rows x K): t0 = e4m3(v), t1 = e4m3(v - t0), t2 = e4m3(v - t0 - t1)
    with v = x * (1/s)."""
    import torch
    amax = x.abs().amax(dim=1, keepdim=True)
    s = torch.where(amax > 0, amax / 448.0, torch.ones_like(amax))
    r = x * (1.0 / s)
    terms = []
    for _ in range(nterms):
        t = r.to(torch.float8_e4m3fn).to(torch.float32)
        terms.append(t.to(torch.float64))
        r = r - t
    return s.to(torch.float64), terms


PAIRS = {"fp8x2": [(1, 0), (0, 1), (0, 0)],
         "fp8x3": [(2, 0), (0, 2), (1, 1), (1, 0), (0, 1), (0, 0)]}


@pytest.mark.parametrize("prec", ["fp8x2", "fp8x3"])
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (200, 300, 100), (1000, 600, 256),
                                   (257, 513, 1000)])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T")])
def test_sgemm_tc_fp8_terms_vs_fp64_reference(cuda, prec, m, n, k, ta, tb):
    """Two- and three-term e4m3 (precisions 5, 6): the tensor cores take the
    products t_i t_j (i + j <= 1, or <= 2) of the scaled operands' terms; the
    FP64 reference forms the same products from the same terms.  The tensor
    core's FP8 sums are not full FP32 (measured up to 2.2e-5 normwise at
    K' = 3K = 336), so the bar is 1e-4 normwise and 1e-3 elementwise for
    K' <= 768 and 1e-3 beyond -- still 40x below the 2^-8 operand error two
    terms leave.  The result must also be much closer to the exact product of
    the FP32 operands than one-term e4m3 (and three terms than two)."""
    import torch
    A = colmajor(torch, m if ta == "N" else k, k if ta == "N" else m, 11 + m, cuda)
    B = colmajor(torch, k if tb == "N" else n, n if tb == "N" else k, 12 + n, cuda)
    C0 = colmajor(torch, m, n, 13 + k, cuda)
    alpha, beta = -1.0, 1.0
    opA = A if ta == "N" else A.t()
    opB = B if tb == "N" else B.t()
    nt = 2 if prec == "fp8x2" else 3
    sa, ta_ = fp8_terms(opA.contiguous(), nt)
    sb, tb_ = fp8_terms(opB.t().contiguous(), nt)
    prod = sa * sum(ta_[i] @ tb_[j].t() for i, j in PAIRS[prec]) * sb.t()
    ref = alpha * prod + beta * C0.to(torch.float64)
    absA, absB = sum(t.abs() for t in ta_), sum(t.abs() for t in tb_)
    bound = abs(alpha) * (sa * (absA @ absB.t()) * sb.t()) + abs(beta) * C0.abs().to(torch.float64)
    C = C0.clone()
    sgemm_tc(prec, ta, tb, alpha, A, B, beta, C)
    err = C.to(torch.float64) - ref
    rel = (err.norm() / ref.norm()).item()
    elem = (err.abs() / bound.clamp_min(1e-30)).max().item()
    kseg = len(PAIRS[prec]) * k
    tol_rel, tol_elem = (1e-4, 1e-3) if kseg <= 768 else (1e-3, 1e-3)
    assert rel <= tol_rel and elem <= tol_elem, (rel, elem)
    # against the exact product of the FP32 operands: one term ~2^-4,
    # two ~2^-8, three ~2^-12 (down to the FP8 summation error at long K')
    exact = alpha * (opA.double() @ opB.double()) + beta * C0.double()
    C1 = C0.clone()
    sgemm_tc("fp8", ta, tb, alpha, A, B, beta, C1)
    e_n = ((C.double() - exact).norm() / exact.norm()).item()
    e_1 = ((C1.double() - exact).norm() / exact.norm()).item()
    if prec == "fp8x2":
        assert e_n <= e_1 / 8 and e_n <= 8e-3, (e_n, e_1)
    else:
        C2 = C0.clone()
        sgemm_tc("fp8x2", ta, tb, alpha, A, B, beta, C2)
        e_2 = ((C2.double() - exact).norm() / exact.norm()).item()
        # (over long K' the FP8 summation error, ~2e-4, is what is left)
        assert e_n <= (e_2 / 4 if kseg <= 768 else e_2) and e_n <= max(5e-4, 2 * tol_rel), (e_n, e_2)
