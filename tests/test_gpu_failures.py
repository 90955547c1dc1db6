"""Failure detection without a GPU fault.

The reference reports failure only through LAPACK's INFO: < 0 for a bad
argument (flens/lapack/interface/src/getrf.cc:22-35), > 0 for the first exactly
zero pivot (flens/lapack/ge/tf2.tcc:123-125).  On top of that the library has
two failure paths of its own, and these tests drive each of them on purpose:

* a device allocation that fails: the host-side hook
  flens_gb300_test_fail_device_allocs makes the library's next cudaMalloc
  fail as an out-of-memory one would.  The calls must return
  FLENS_GB300_ERR_ALLOC (INFO for the Fortran-ABI symbols) with a message,
  and work again once memory is available;
* a bounded device-side wait that gives up: flens_gb300_test_stall_next_chain
  makes the first block of the next chained triangular solve wait, with a
  short spin limit, for a flag that nothing sets.  Every block gives up and
  returns; flens_gb300_sync reports FLENS_GB300_ERR_TIMEOUT, and the same
  context then solves correctly.  Nothing faults, traps or waits unbounded.
"""
import ctypes
import threading

import numpy as np
import pytest

import flens_gb300 as fg
import oracle

pytestmark = pytest.mark.gpu


def _fail_next(k):
    f = fg.lib().flens_gb300_test_fail_device_allocs
    f.argtypes = [ctypes.c_int]
    f.restype = None
    f(k)


def _lu(cuda, n, seed):
    import torch
    A0 = oracle.uniform(seed, n, n)
    A0[np.arange(n), np.arange(n)] += n / 4.0
    return A0, fg.to_colmajor(torch.from_numpy(A0).to(cuda))


def test_alloc_failure_device_api_then_recovers(cuda):
    import torch
    n = 256
    A0, dA = _lu(cuda, n, 71)
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    s = torch.cuda.Stream()                       # a stream without a workspace yet
    s.wait_stream(torch.cuda.current_stream())    # dA, ipiv, info are made there
    _fail_next(1)
    try:
        with pytest.raises(fg.FlensGB300Error) as e:
            fg.dgetrf_dev(dA, ipiv, info, stream=s)
        assert e.value.code == fg.ERR_ALLOC
        assert "cudaMalloc" in str(e.value)
    finally:
        _fail_next(0)
    fg.dgetrf_dev(dA, ipiv, info, stream=s)
    b0 = oracle.uniform(76, n, 1)
    b = fg.to_colmajor(torch.from_numpy(b0).to(cuda))
    s.wait_stream(torch.cuda.current_stream())
    fg.dgetrs_dev("N", dA, ipiv, b, stream=s)
    fg.sync(s)
    assert int(info.item()) == 0
    assert oracle.normwise_rel(b.cpu().numpy(), np.linalg.solve(A0, b0)) <= 1e-12


def test_alloc_failure_host_dgesv_info(cuda):
    # the Fortran-ABI dgesv_ has INFO: the allocation failure comes back there.
    # A new host thread has no staging buffers yet, so its first call allocates.
    n = 200
    A = oracle.uniform(72, n, n)
    A[np.arange(n), np.arange(n)] += n / 4.0
    B = oracle.uniform(73, n, 2)
    out = {}

    def run():
        _fail_next(1)
        try:
            out["first"] = fg.dgesv(A.copy(order="F"), B.copy(order="F"))[1]
            out["msg"] = fg.last_error()
        finally:
            _fail_next(0)
        Bx = B.copy(order="F")
        out["second"] = fg.dgesv(A.copy(order="F"), Bx)[1]
        out["x"] = Bx

    t = threading.Thread(target=run)
    t.start()
    t.join()
    assert out["first"] == fg.ERR_ALLOC
    assert "cudaMalloc" in out["msg"]
    assert out["second"] == 0
    x = np.linalg.solve(A, B)
    assert oracle.normwise_rel(out["x"], x) <= 1e-12


def test_alloc_failure_split_gemm(cuda):
    import torch
    m = n = k = 192
    g = torch.Generator(device=cuda)
    g.manual_seed(3)
    A = fg.to_colmajor(torch.rand((m, k), generator=g, dtype=torch.float64, device=cuda))
    B = fg.to_colmajor(torch.rand((k, n), generator=g, dtype=torch.float64, device=cuda))
    C = fg.colmajor_empty(m, n, device=cuda)
    C.zero_()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())    # A, B, C are made there
    _fail_next(1)
    try:
        with pytest.raises(fg.FlensGB300Error) as e:
            fg.dgemm_split_dev("N", "N", 1.0, A, B, 0.0, C, stream=s)
        assert e.value.code == fg.ERR_ALLOC
    finally:
        _fail_next(0)
    fg.dgemm_split_dev("N", "N", 1.0, A, B, 0.0, C, stream=s)
    fg.sync(s)                                    # C is read on the current stream below
    ref = A @ B
    assert ((C - ref).abs().max() / ref.abs().max()).item() <= 1e-13


def test_alloc_failure_batched_plan(cuda, monkeypatch):
    import torch
    from test_gpu_batched import plan_fn
    sizes, ks = [20, 70], [1, 4]
    mats = [fg.to_colmajor(torch.rand((n, n), dtype=torch.float64, device=cuda) + n * torch.eye(
        n, dtype=torch.float64, device=cuda)) for n in sizes]
    rhs = [fg.to_colmajor(torch.rand((n, k), dtype=torch.float64, device=cuda))
           for n, k in zip(sizes, ks)]
    count = len(sizes)
    n = np.array(sizes, dtype=np.int32)
    k = np.array(ks, dtype=np.int32)
    ipivs = [torch.zeros(x, dtype=torch.int32, device=cuda) for x in sizes]
    pa = np.array([t.data_ptr() for t in mats], dtype=np.uint64)
    pb = np.array([t.data_ptr() for t in rhs], dtype=np.uint64)
    pp = np.array([t.data_ptr() for t in ipivs], dtype=np.uint64)
    info = torch.zeros(count, dtype=torch.int32, device=cuda)
    iters = torch.zeros(count, dtype=torch.int32, device=cuda)
    berr = torch.zeros(count, dtype=torch.float64, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    plan = ctypes.c_void_p()
    f = plan_fn()
    args = (count, n.ctypes.data, k.ctypes.data, pa.ctypes.data, n.ctypes.data, pp.ctypes.data,
            pb.ctypes.data, n.ctypes.data, info.data_ptr(), 0, iters.data_ptr(), berr.data_ptr(),
            10, stream, ctypes.byref(plan))
    monkeypatch.setenv("FLENS_GB300_BATCH_TUNE", "0")    # the plan's own allocations first
    _fail_next(1)
    try:
        st = f(*args)
    finally:
        _fail_next(0)
    assert st == fg.ERR_ALLOC
    assert "alloc" in fg.last_error()
    assert f(*args) == 0, fg.last_error()
    assert fg.lib().flens_gb300_batched_execute(plan, stream) == 0
    fg.lib().flens_gb300_batched_destroy(plan)
    fg.sync()
    assert info.cpu().numpy().tolist() == [0, 0]


def test_bounded_wait_timeout_then_healthy(cuda):
    import torch
    n = 500                                        # 8 blocks: the chained solve
    A0, dA = _lu(cuda, n, 74)
    ipiv = torch.zeros(n, dtype=torch.int32, device=cuda)
    info = torch.zeros(1, dtype=torch.int32, device=cuda)
    fg.dgetrf_dev(dA, ipiv, info)
    fg.sync()
    b0 = oracle.uniform(75, n, 1)
    stall = fg.lib().flens_gb300_test_stall_next_chain
    stall.argtypes = [ctypes.c_uint]
    stall.restype = None
    stall(4000)                                    # a few hundred microseconds of spinning
    b = fg.to_colmajor(torch.from_numpy(b0).to(cuda))
    fg.dgetrs_dev("N", dA, ipiv, b)
    with pytest.raises(fg.FlensGB300Error) as e:
        fg.sync()
    assert e.value.code == fg.ERR_TIMEOUT
    assert "timed out" in str(e.value)
    # the status word was read and cleared; the context still works
    b = fg.to_colmajor(torch.from_numpy(b0).to(cuda))
    fg.dgetrs_dev("N", dA, ipiv, b)
    fg.sync()
    x = np.linalg.solve(A0, b0)
    assert oracle.normwise_rel(b.cpu().numpy(), x) <= 1e-12


def test_mixed_inverse_preconditioner_falls_back_without_memory(cuda):
    # BF16 factors at n >= 2048 take GMRES with explicit inverses of L and U,
    # whose workspace is requested first; when that allocation fails the
    # solve must fall back to the chained preconditioner and still converge.
    # A GMRES-IR solve with 3xTF32 factors on the same (fresh) stream first
    # sizes every other workspace, so the next allocation is the inverses'.
    import torch
    from test_gpu_mixed import make_system, backward_error, PREC, SOLVER, EPS
    n = 2048
    A, b, x = make_system(cuda, n, 1e2, 1, 31)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())    # A and b are made there
    f = fg.lib().flens_gb300_dgesv_mixed
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]

    def solve(prec, solver):
        X = fg.colmajor_empty(n, 1, device=cuda)
        it, be, inf = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        st = f(n, 1, A.data_ptr(), n, b.data_ptr(), n, X.data_ptr(), n, PREC[prec], SOLVER[solver],
               30, 0.0, ctypes.byref(it), ctypes.byref(be), ctypes.byref(inf),
               ctypes.c_void_p(s.cuda_stream))
        s.synchronize()
        return st, X, it.value

    st, X, it = solve("fp32", "gmres")
    assert st == 0, fg.last_error()
    count = fg.lib().flens_gb300_device_alloc_count
    count.restype = ctypes.c_longlong
    before = count()
    _fail_next(1)
    try:
        st, X, it = solve("bf16", "auto")
    finally:
        _fail_next(0)
    assert st == 0, (st, fg.last_error(), it)
    assert count() == before                    # the one allocation it tried was refused
    assert backward_error(A, X, b) <= 10 * n * EPS
