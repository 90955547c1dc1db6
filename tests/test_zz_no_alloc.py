"""flens_gb300_dgetrs_noalloc: the solve for callers that cannot allocate.

Some callers must not call cudaMalloc once they are running (a fixed device
memory budget reserved at start-up, a memory pool owned by another framework,
a process that forbids device allocation on its serving path).  This entry
point solves from dgetrf's factors like flens_gb300_dgetrs but keeps its
scratch in a fixed array inside the library.  The test calls it through the
C ABI, twice in a row (the array keeps the previous call's contents), and
checks each result against flens_gb300_dgetrs within the solve tolerance the
other LU tests use.  This file is collected last so that a failure here comes
after every other test has run; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import flens_gb300 as fg
import oracle

pytestmark = pytest.mark.gpu

SOLVE_TOL = 1e-12


def _factor(cuda, n, seed):
    import torch
    A0 = oracle.uniform(seed, n, n)
    dA = fg.to_colmajor(torch.from_numpy(A0).to(cuda))
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_dev(dA, ipiv, info)
    fg.sync()
    assert int(info.item()) == 0
    return dA, ipiv


def _noalloc(trans, LU, ipiv, B):
    import torch
    n = LU.shape[0]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return fg.lib().flens_gb300_dgetrs_noalloc(trans.encode(), n, B.shape[1], LU.data_ptr(),
                                               LU.stride(1), ipiv.data_ptr(), B.data_ptr(),
                                               B.stride(1), stream)


@pytest.mark.parametrize("trans", "NT")
def test_noalloc_matches_dgetrs_two_calls(cuda, trans):
    import torch
    n = 300
    LU, ipiv = _factor(cuda, n, 4242)
    for call, nrhs in enumerate((5, 3)):
        B0 = oracle.uniform(100 + call, n, nrhs)
        want = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        got = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        fg.dgetrs_dev(trans, LU, ipiv, want)
        assert _noalloc(trans, LU, ipiv, got) == 0, fg.last_error()
        fg.sync()
        err = oracle.normwise_rel(got.cpu().numpy(), want.cpu().numpy())
        assert err <= SOLVE_TOL, (call, err)


def test_noalloc_rejects_oversize(cuda):
    import torch
    n = 8192
    LU = fg.colmajor_empty(n, n, device=cuda)
    ipiv = torch.ones(n, dtype=torch.int32, device=cuda)
    B = fg.colmajor_empty(n, 128, device=cuda)      # 8 MiB of right-hand sides: too many
    assert _noalloc("N", LU, ipiv, B) == fg.ERR_UNSUPPORTED
    assert "scratch" in fg.last_error()
