"""Batched uneven-size dgesv in one persistent launch (graph replay) against
the oracle, matrix by matrix.

Each matrix is the reference's dgesv (flens/lapack/ge/sv.tcc:58-77): the bar
is identical pivots and INFO on well-separated inputs, solutions within 1e-12
normwise of the oracle's, B untouched when INFO > 0.  The mixed variant (FP32
LU + FP64 refinement) must reach a normwise backward error <= 10 n eps64.
"""
import ctypes

import numpy as np
import pytest

import flens_gb300 as fg
import oracle

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def plan_fn():
    L = fg.lib()
    f = L.flens_gb300_dgesv_batched_plan
    vp = ctypes.c_void_p
    f.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, vp, vp, ctypes.c_int,
                  vp, ctypes.POINTER(ctypes.c_void_p)]
    f.restype = ctypes.c_int
    L.flens_gb300_batched_execute.argtypes = [vp, vp]
    L.flens_gb300_batched_execute.restype = ctypes.c_int
    L.flens_gb300_batched_destroy.argtypes = [vp]
    L.flens_gb300_batched_team.argtypes = [vp, ctypes.c_int]
    L.flens_gb300_batched_team.restype = ctypes.c_int
    L.flens_gb300_batched_panel.argtypes = [vp, ctypes.c_int]
    L.flens_gb300_batched_panel.restype = ctypes.c_int
    return f


def make_batch(cuda, sizes, ks, seed, singular=(), shift=True):
    import torch
    mats, rhs, host = [], [], []
    for i, (n, k) in enumerate(zip(sizes, ks)):
        A = oracle.uniform(seed + 2 * i, n, n)
        if shift:
            A[np.arange(n), np.arange(n)] += n / 4.0
        if i in singular:
            A[:, n // 2] = 0.0
        B = oracle.uniform(seed + 2 * i + 1, n, k)
        host.append((A, B))
        mats.append(fg.to_colmajor(torch.from_numpy(A).to(cuda)))
        rhs.append(fg.to_colmajor(torch.from_numpy(B).to(cuda)))
    return mats, rhs, host


def run_batched(cuda, mats, rhs, precision, execs=1):
    import torch
    count = len(mats)
    n = np.array([m.shape[0] for m in mats], dtype=np.int32)
    k = np.array([b.shape[1] for b in rhs], dtype=np.int32)
    lda = np.maximum(n, 1).astype(np.int32)
    ipivs = [torch.zeros(max(1, int(x)), dtype=torch.int32, device=cuda) for x in n]
    pa = np.array([m.data_ptr() for m in mats], dtype=np.uint64)
    pb = np.array([b.data_ptr() for b in rhs], dtype=np.uint64)
    pp = np.array([p.data_ptr() for p in ipivs], dtype=np.uint64)
    info = torch.full((count,), -7, dtype=torch.int32, device=cuda)
    iters = torch.zeros(count, dtype=torch.int32, device=cuda)
    berr = torch.zeros(count, dtype=torch.float64, device=cuda)
    plan = ctypes.c_void_p()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = plan_fn()(count, n.ctypes.data, k.ctypes.data, pa.ctypes.data, lda.ctypes.data,
                   pp.ctypes.data, pb.ctypes.data, lda.ctypes.data, info.data_ptr(), precision,
                   iters.data_ptr(), berr.data_ptr(), 10, stream, ctypes.byref(plan))
    assert st == 0, fg.last_error()
    for _ in range(execs):
        assert fg.lib().flens_gb300_batched_execute(plan, stream) == 0
    torch.cuda.synchronize()
    teams = [fg.lib().flens_gb300_batched_team(plan, b) for b in range(16)]
    teams = teams[:teams.index(-1)]
    panels = [fg.lib().flens_gb300_batched_panel(plan, b) for b in range(len(teams) + 1)]
    assert panels[-1] == -1 and all(p in (8, 16) for p in panels[:-1])
    # the blocked path's panels fit the team's share of 216 KB of shared memory
    # for every bucket bound up to 864
    for b, (t, p) in enumerate(zip(teams, panels)):
        if b < len(BUCKET_MAX) and BUCKET_MAX[b] > 64:
            share = 216 * 1024 // (256 // t)
            fits_shared = (BUCKET_MAX[b] ** 2 + BUCKET_MAX[b] * 16) * 8 <= share
            assert fits_shared or 2 * BUCKET_MAX[b] * p * 8 <= share or t == 256, (b, t, p)
    fg.lib().flens_gb300_batched_destroy(plan)
    fg.sync()
    # (team size, panel width) per bucket
    return ipivs, info.cpu().numpy(), iters.cpu().numpy(), berr.cpu().numpy(), list(zip(teams, panels))


SIZES = [1, 8, 9, 16, 17, 31, 32, 33, 48, 64, 65, 100, 128, 129, 160, 200, 256, 300, 13, 40]
KS = [1, 4, 16, 1, 4, 16, 1, 4, 16, 1, 4, 16, 1, 4, 16, 1, 4, 16, 4, 1]


def test_batched_fp64_vs_oracle(cuda, port):
    mats, rhs, host = make_batch(cuda, SIZES, KS, 500, singular=(18,))
    B0 = [b.clone() for b in rhs]
    ipivs, info, iters, berr, teams = run_batched(cuda, mats, rhs, 0)
    for i, (A0, Bh) in enumerate(host):
        A1, B1 = A0.copy(order="F"), Bh.copy(order="F")
        pivr, infor = port.dgesv(A1, B1)
        assert info[i] == infor, (i, SIZES[i], info[i], infor)
        n = SIZES[i]
        assert np.array_equal(ipivs[i].cpu().numpy()[:n], pivr), i
        if infor == 0:
            assert oracle.normwise_rel(rhs[i].cpu().numpy(), B1) <= 1e-12, i
            assert oracle.lu_backward_error(A0, mats[i].cpu().numpy(), pivr) <= 10.0
        else:
            assert np.array_equal(rhs[i].cpu().numpy(), B0[i].cpu().numpy())   # no solve
    assert all(t in (32, 64, 128, 256) and p in (8, 16) for t, p in teams)


def test_batched_blocked_path_pivoting(cuda, port):
    # n > 160 does not fit a team's shared memory: the blocked factorisation
    # in global memory; unshifted inputs so that it interchanges rows
    # (the solves stage the right-hand sides in shared memory in column
    # groups of 1, 4 or 8; k = 9 leaves a ragged group, k = 40 may exceed
    # the team's share and solve in global memory)
    sizes, ks = [161, 200, 333, 512, 250, 300, 400], [1, 4, 16, 1, 3, 9, 40]
    mats, rhs, host = make_batch(cuda, sizes, ks, 1500, singular=(4,), shift=False)
    B0 = [b.clone() for b in rhs]
    ipivs, info, _, _, _ = run_batched(cuda, mats, rhs, 0)
    for i, (A0, Bh) in enumerate(host):
        A1, B1 = A0.copy(order="F"), Bh.copy(order="F")
        pivr, infor = port.dgesv(A1, B1)
        n = sizes[i]
        assert info[i] == infor, (i, n, info[i], infor)
        assert np.array_equal(ipivs[i].cpu().numpy()[:n], pivr), i
        assert oracle.lu_backward_error(A0, mats[i].cpu().numpy(), pivr) <= 10.0, i
        if infor == 0:
            assert oracle.normwise_rel(rhs[i].cpu().numpy(), B1) <= 1e-10, i
        else:
            assert np.array_equal(rhs[i].cpu().numpy(), B0[i].cpu().numpy())


# upper bounds of the plan's size buckets (flens_gb300_batched_team)
BUCKET_MAX = [16, 32, 48, 64, 108, 216, 320, 432, 864]


def bucket_of(n):
    return next((b for b, m in enumerate(BUCKET_MAX) if n <= m), len(BUCKET_MAX))


def test_batched_team_sizes_fit_shared_memory(cuda, port):
    # a bucket's (team size, panel width) keeps its largest matrix in shared
    # memory or on the blocked path.  With 16-column panels, 2 teams per CTA
    # (T = 128) hold the panels of n <= 432 and only one team (T = 256) those
    # of n = 433..864; 8-column panels halve that need.
    sizes, ks = [500, 432, 400, 216, 200, 108, 100], [4, 1, 16, 4, 1, 16, 4]
    mats, rhs, host = make_batch(cuda, sizes, ks, 2100)
    ipivs, info, _, _, teams = run_batched(cuda, mats, rhs, 0)
    assert len(teams) == len(BUCKET_MAX) + 1
    feasible = lambda t, p, n: 2 * n * p * 8 <= 216 * 1024 // (256 // t)
    for n in (500, 432, 400, 216, 200):
        t, p = teams[bucket_of(n)]
        assert feasible(t, p, BUCKET_MAX[bucket_of(n)]), (n, t, p)
    assert teams[bucket_of(216)][0] in (64, 128, 256)
    assert teams[bucket_of(108)][0] in (32, 64, 128, 256)
    for i, (A0, Bh) in enumerate(host):
        A1, B1 = A0.copy(order="F"), Bh.copy(order="F")
        pivr, infor = port.dgesv(A1, B1)
        assert info[i] == infor == 0
        assert np.array_equal(ipivs[i].cpu().numpy()[:sizes[i]], pivr), i
        assert oracle.normwise_rel(rhs[i].cpu().numpy(), B1) <= 1e-12, i


def test_batched_graph_replay(cuda, port):
    # the plan's graph replays the same launch: second execution on fresh data
    import torch
    mats, rhs, host = make_batch(cuda, SIZES[:12], KS[:12], 700)
    ipivs, info, _, _, _ = run_batched(cuda, mats, rhs, 0, execs=1)
    assert (info == 0).all()
    for i, (A0, Bh) in enumerate(host):
        A1, B1 = A0.copy(order="F"), Bh.copy(order="F")
        port.dgesv(A1, B1)
        assert oracle.normwise_rel(rhs[i].cpu().numpy(), B1) <= 1e-12


def test_batched_mixed_refinement(cuda):
    import torch
    sizes = [8, 20, 33, 64, 100, 128, 200, 17, 50, 90]
    ks = [1, 4, 16, 1, 4, 16, 1, 4, 16, 1]
    mats, rhs, host = make_batch(cuda, sizes, ks, 900)
    ipivs, info, iters, berr, teams = run_batched(cuda, mats, rhs, 1)
    assert (info == 0).all(), info
    for i, (A0, Bh) in enumerate(host):
        n = sizes[i]
        X = rhs[i].cpu().numpy()
        R = Bh - A0 @ X
        be = (np.abs(R).max(0) / (np.abs(A0).sum(1).max() * np.abs(X).max(0) + np.abs(Bh).max(0))).max()
        assert be <= 10 * n * EPS, (i, n, be, iters[i])
        if iters[i] >= 0:
            # the FP32 path: A untouched, its own backward error reported
            assert berr[i] <= 10 * n * EPS
            np.testing.assert_array_equal(mats[i].cpu().numpy(), A0)
        else:
            # FP32 working set too large for the team: the FP64 path, A <- LU
            assert oracle.lu_backward_error(A0, mats[i].cpu().numpy(), ipivs[i].cpu().numpy()[:n]) <= 10.0


def test_batched_mixed_refinement_blocked_fp32(cuda, port):
    # matrices whose FP32 working set does not fit a team's shared memory:
    # FP32 factors of a copy of A in the plan's pool (blocked LU, panels in
    # shared memory), FP64 refinement against the untouched A; k = 40 exceeds
    # the 32 columns the refinement tracks and takes the FP64 path
    sizes = [170, 257, 300, 431, 512, 333, 480]
    ks = [1, 4, 16, 3, 1, 9, 40]
    mats, rhs, host = make_batch(cuda, sizes, ks, 3100)
    ipivs, info, iters, berr, teams = run_batched(cuda, mats, rhs, 1)
    assert (info == 0).all(), info
    for i, (A0, Bh) in enumerate(host):
        n = sizes[i]
        X = rhs[i].cpu().numpy()
        R = Bh - A0 @ X
        be = (np.abs(R).max(0) / (np.abs(A0).sum(1).max() * np.abs(X).max(0) + np.abs(Bh).max(0))).max()
        assert be <= 10 * n * EPS, (i, n, be, iters[i])
        A1, B1 = A0.copy(order="F"), Bh.copy(order="F")
        pivr, _ = port.dgesv(A1, B1)
        assert oracle.normwise_rel(X, B1) <= 1e-12, i
        if ks[i] <= 32:
            # the FP32 path ran: A untouched, refinement steps and backward error reported
            assert iters[i] >= 0, (i, iters[i])
            assert berr[i] <= 10 * n * EPS
            np.testing.assert_array_equal(mats[i].cpu().numpy(), A0)
            # FP64 pivot search on the FP32 factors of a diagonally dominant A
            assert np.array_equal(ipivs[i].cpu().numpy()[:n], pivr), i
        else:
            assert iters[i] == -1
            assert oracle.lu_backward_error(A0, mats[i].cpu().numpy(), ipivs[i].cpu().numpy()[:n]) <= 10.0


def test_batched_mixed_many_buckets_no_slot_sharing(cuda):
    # many matrices in buckets with different team sizes: CTAs move through
    # the buckets independently, so the pool slots of the blocked FP32 path
    # must not depend on the bucket's team size (a shared slot gives wrong
    # or non-finite solutions for a few matrices, different from run to run)
    import torch
    sizes = [100, 200, 300, 420, 500, 96, 330] * 90
    ks = [16, 4, 16, 16, 1, 16, 16] * 90
    mats, rhs, host = make_batch(cuda, sizes, ks, 4100)
    ipivs, info, iters, berr, teams = run_batched(cuda, mats, rhs, 1)
    assert (info == 0).all()
    assert (iters >= 0).all()
    for i, (A0, Bh) in enumerate(host):
        n = sizes[i]
        A = torch.from_numpy(A0).to(cuda)
        B = torch.from_numpy(Bh).to(cuda)
        X = rhs[i]
        assert torch.isfinite(X).all(), (i, n)
        R = B - A @ X
        den = A.abs().sum(1).max() * X.abs().amax(0) + B.abs().amax(0)
        be = (R.abs().amax(0) / den).max().item()
        assert be <= 10 * n * EPS, (i, n, ks[i], be, iters[i])


def test_batched_auto_precision_per_matrix(cuda, port):
    # precision 2: FP32 LU + FP64 refinement only where it is faster (n >= 256
    # and k <= n/64), the FP64 path (iters = -1, A <- LU) for the rest
    sizes = [16, 100, 200, 256, 300, 512, 512, 300, 64]
    ks = [4, 1, 4, 4, 4, 1, 16, 5, 1]
    mats, rhs, host = make_batch(cuda, sizes, ks, 5200)
    ipivs, info, iters, berr, teams = run_batched(cuda, mats, rhs, 2)
    assert (info == 0).all(), info
    for i, (A0, Bh) in enumerate(host):
        n, k = sizes[i], ks[i]
        X = rhs[i].cpu().numpy()
        A1, B1 = A0.copy(order="F"), Bh.copy(order="F")
        pivr, _ = port.dgesv(A1, B1)
        assert oracle.normwise_rel(X, B1) <= 1e-12, i
        if n >= 256 and 64 * k <= n:
            assert iters[i] >= 0, (i, n, k, iters[i])
            assert berr[i] <= 10 * n * EPS
            np.testing.assert_array_equal(mats[i].cpu().numpy(), A0)
        else:
            assert iters[i] == -1, (i, n, k, iters[i])
            assert np.array_equal(ipivs[i].cpu().numpy()[:n], pivr), i
            assert oracle.lu_backward_error(A0, mats[i].cpu().numpy(), ipivs[i].cpu().numpy()[:n]) <= 10.0


def test_batched_unshifted_n512_pivots(cuda, port):
    # eight unshifted 512 x 512 systems (the blocked global-memory path, about
    # 500 interchanges each): pivots entry by entry on every pivot search whose
    # two largest |candidates| differ by more than 1e-10 relative
    sizes, ks = [512] * 8, [1, 4, 16, 1, 4, 16, 1, 4]
    mats, rhs, host = make_batch(cuda, sizes, ks, 2500, shift=False)
    ipivs, info, _, _, _ = run_batched(cuda, mats, rhs, 0)
    for i, (A0, Bh) in enumerate(host):
        pivr, infor, gap = port.dgetrf_gaps(A0.copy(order="F"))
        assert info[i] == infor == 0
        piv = ipivs[i].cpu().numpy()[:512]
        sep = gap > 1e-10
        assert sep.mean() > 0.99
        assert np.array_equal(piv[sep], pivr[sep]), i
        assert np.count_nonzero(pivr != np.arange(1, 513)) > 400
        x = np.linalg.solve(A0, Bh)
        assert oracle.normwise_rel(rhs[i].cpu().numpy(), x) <= 1e-10, i
