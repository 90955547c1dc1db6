"""flens_gb300_dgetrs_noalloc: the solve for callers that cannot allocate.

Some callers must not call cudaMalloc once they are running (a fixed device
memory budget reserved at start-up, a memory pool owned by another framework,
a process that forbids device allocation on its serving path).  This entry
point solves from dgetrf's factors like flens_gb300_dgetrs but keeps all of its
scratch in a fixed array inside the library.

The tests call it through the C ABI first on a stream the library has never
seen, where flens_gb300_dgetrs would create a workspace, with 1 to 4
right-hand sides (the chained solve, which needs ready flags and a status
word), and check with the library's own allocation counter that it made no
device allocation.  Each result is compared with flens_gb300_dgetrs (run on a
different stream) within the solve tolerance the other LU tests use, on two
calls in a row (the array keeps the previous call's contents).  This file is
collected last so that a failure here comes after every other test has run; it
also passes on its own in a fresh process.
"""
import ctypes

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


def _noalloc(trans, LU, ipiv, B, stream):
    n = LU.shape[0]
    return fg.lib().flens_gb300_dgetrs_noalloc(trans.encode(), n, B.shape[1], LU.data_ptr(),
                                               LU.stride(1), ipiv.data_ptr(), B.data_ptr(),
                                               max(B.stride(1), n), ctypes.c_void_p(stream.cuda_stream))


def _allocs():
    f = fg.lib().flens_gb300_device_alloc_count
    f.restype = ctypes.c_longlong
    return int(f())


@pytest.mark.parametrize("trans", "NT")
def test_noalloc_fresh_stream_no_allocation_two_calls(cuda, trans):
    import torch
    n = 300                                        # 5 blocks of 64: the chained solve
    LU, ipiv = _factor(cuda, n, 4242)
    fresh = torch.cuda.Stream()                    # no library workspace exists for it
    for call, nrhs in enumerate((3, 4)):
        B0 = oracle.uniform(100 + call, n, nrhs)
        want = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        got = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        torch.cuda.synchronize()
        before = _allocs()
        assert _noalloc(trans, LU, ipiv, got, fresh) == 0, fg.last_error()
        fresh.synchronize()
        assert _allocs() == before, "flens_gb300_dgetrs_noalloc allocated device memory"
        fg.dgetrs_dev(trans, LU, ipiv, want)       # the library's current-stream path
        fg.sync()
        err = oracle.normwise_rel(got.cpu().numpy(), want.cpu().numpy())
        assert err <= SOLVE_TOL, (call, err)


@pytest.mark.parametrize("trans", "NT")
def test_noalloc_many_rhs_two_calls(cuda, trans):
    import torch
    n = 300
    LU, ipiv = _factor(cuda, n, 4343)
    stream = torch.cuda.current_stream()
    for call, nrhs in enumerate((5, 17)):         # the blocked solve path
        B0 = oracle.uniform(200 + call, n, nrhs)
        want = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        got = fg.to_colmajor(torch.from_numpy(B0).to(cuda))
        before = _allocs()
        assert _noalloc(trans, LU, ipiv, got, stream) == 0, fg.last_error()
        stream.synchronize()
        assert _allocs() == before
        fg.dgetrs_dev(trans, LU, ipiv, want)
        fg.sync()
        err = oracle.normwise_rel(got.cpu().numpy(), want.cpu().numpy())
        assert err <= SOLVE_TOL, (call, err)


def test_noalloc_rejects_oversize(cuda):
    import torch
    n = 8192
    LU = fg.colmajor_empty(n, n, device=cuda)
    ipiv = torch.ones(n, dtype=torch.int32, device=cuda)
    B = fg.colmajor_empty(n, 128, device=cuda)      # 8 MiB of right-hand sides: too many
    assert _noalloc("N", LU, ipiv, B, torch.cuda.current_stream()) == fg.ERR_UNSUPPORTED
    assert "scratch" in fg.last_error()
