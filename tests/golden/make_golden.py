"""Generate the golden fixtures in this directory from the REFERENCE itself.

Runs the reference's own Fortran-ABI shims (dgemm_, dtrsm_, dsyrk_, dtrmm_,
dsymm_, dsyr2k_, dgetrf_, dgetrs_, dgesv_, dgetri_, dtrtri_, dpotrf_, dpotrs_,
dposv_, dgecon_, dgerfs_, dgeequ_, dlaqge_, dgesvx_ compiled
from the FLENS sources into
oracle/_ref/libflens_ref.so by
``make -C oracle ref``) on seeded inputs and stores the outputs.  Inputs come
from ``oracle.splitmix_uniform(seed, m, n)`` (integer hashing, identical on
every machine), so only seeds and outputs are stored.  The fixtures travel
with the repository: machines without the reference sources (the GPU host)
still pin the oracle and check the GPU library against the reference's own
results.

    python tests/golden/make_golden.py            # small fixtures (seconds)
    python tests/golden/make_golden.py --large    # + the n=8192 LU pivots (minutes)
    python tests/golden/make_golden.py --no-small --pivots   # unshifted n=2048/4096 pivots
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

U = oracle.splitmix_uniform


# ----------------------------------------------------------- case lists --
# Shared with the tests: each case is (name, parameters); inputs are rebuilt
# from the parameters with gemm_inputs / trsm_inputs / lu_input.
def gemm_case_list():
    cases = []
    for (m, n, k) in [(0, 3, 2), (1, 1, 1), (3, 0, 5), (4, 3, 0)]:
        cases.append((m, n, k, "N", "N", 1.5, 0.5))
    for ta in "NT":
        for tb in "NT":
            cases.append((7, 31, 63, ta, tb, 1.5, 0.5))
    for (a, b) in [(0.0, 1.3), (0.7, 0.0), (1.0, 1.0), (-1.0, 1.0)]:
        cases.append((7, 31, 63, "N", "N", a, b))
    for ta in "NTC":
        for tb in "NTC":
            cases.append((65, 33, 130, ta, tb, 1.5, 0.5))
    return [(f"gemm{i:03d}", c) for i, c in enumerate(cases)]


def gemm_inputs(i, m, n, k, ta, tb):
    s = 1000 + 10 * i
    A = U(s, m if ta == "N" else k, k if ta == "N" else m)
    B = U(s + 1, k if tb == "N" else n, n if tb == "N" else k)
    C = U(s + 2, m, n)
    return A, B, C


def trsm_case_list():
    cases = []
    for (m, n) in [(33, 17), (70, 3)]:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        cases.append((m, n, side, uplo, ta, diag, 0.7))
    cases.append((33, 17, "L", "L", "C", "N", 1.0))
    cases.append((1, 5, "L", "U", "N", "N", -2.0))
    return [(f"trsm{i:03d}", c) for i, c in enumerate(cases)]


def trsm_inputs(i, m, n, side):
    s = 5000 + 10 * i
    ka = m if side == "L" else n
    A = U(s, ka, ka)
    A[np.arange(ka), np.arange(ka)] += 2.0 + ka / 4.0
    B = U(s + 1, m, n)
    return A, B


def lu_case_list():
    cases = []
    for (m, n) in [(1, 1), (2, 2), (4, 4), (10, 7), (7, 10), (31, 31), (64, 64), (65, 65),
                   (100, 80), (80, 100), (129, 129)]:
        for kind in ("uniform", "shifted"):
            cases.append((m, n, kind))
    return [(f"lu{i:03d}", c) for i, c in enumerate(cases)]


def lu_input(i, m, n, kind):
    A = U(9000 + 10 * i, m, n)
    if kind == "shifted":
        d = min(m, n)
        A[np.arange(d), np.arange(d)] += max(m, n) / 4.0
    return A


def lu_rhs(i, n):
    return U(9000 + 10 * i + 1, n, 3)


def singular_input():
    A = U(7777, 12, 12)
    A[:, 2] = 0.0
    return A


def baby_problem():
    """The 4x4 system of the reference example flens/examples/lapack-gesv.cc:39-47."""
    A = np.asfortranarray([[2, 3, -1, 0], [-6, -5, 0, 2], [2, -5, 6, -6], [4, 6, 2, -3]],
                          dtype=np.float64)
    b = np.asfortranarray([[20], [-33], [-43], [49]], dtype=np.float64)
    return A, b


def syrk_case_list():
    cases = []
    for (n, k) in [(0, 3), (5, 0), (7, 9), (40, 33), (65, 130)]:
        for uplo in "LU":
            for tr in "NTC":
                cases.append((n, k, uplo, tr, 1.5, 0.5))
    for (a, b) in [(-1.0, 1.0), (0.0, 2.0), (2.0, 0.0)]:
        cases.append((40, 33, "L", "N", a, b))
    return [(f"syrk{i:03d}", c) for i, c in enumerate(cases)]


def syrk_inputs(i, n, k, tr):
    s = 11000 + 10 * i
    A = U(s, n if tr == "N" else k, k if tr == "N" else n)
    C = U(s + 1, n, n)
    return A, C


def trmm_case_list():
    cases = []
    for (m, n) in [(33, 17), (70, 3), (1, 5)]:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        cases.append((m, n, side, uplo, ta, diag, 0.7))
    cases.append((33, 17, "L", "L", "C", "N", 1.0))
    cases.append((0, 4, "L", "U", "N", "N", 1.0))
    return [(f"trmm{i:03d}", c) for i, c in enumerate(cases)]


def trmm_inputs(i, m, n, side):
    s = 15000 + 10 * i
    ka = m if side == "L" else n
    return U(s, ka, ka), U(s + 1, m, n)


def symm_case_list():
    cases = []
    for (m, n) in [(33, 17), (70, 3), (1, 5), (0, 4)]:
        for side in "LR":
            for uplo in "UL":
                cases.append((m, n, side, uplo, 1.5, 0.5))
    for (a, b) in [(-1.0, 1.0), (0.0, 2.0), (2.0, 0.0)]:
        cases.append((33, 17, "L", "L", a, b))
    return [(f"symm{i:03d}", c) for i, c in enumerate(cases)]


def symm_inputs(i, m, n, side):
    s = 17000 + 10 * i
    ka = m if side == "L" else n
    return U(s, ka, ka), U(s + 1, m, n), U(s + 2, m, n)


def syr2k_case_list():
    cases = []
    for (n, k) in [(0, 3), (5, 0), (7, 9), (40, 33)]:
        for uplo in "LU":
            for tr in "NTC":
                cases.append((n, k, uplo, tr, 1.5, 0.5))
    for (a, b) in [(-1.0, 1.0), (0.0, 2.0)]:
        cases.append((40, 33, "U", "N", a, b))
    return [(f"syr2k{i:03d}", c) for i, c in enumerate(cases)]


def syr2k_inputs(i, n, k, tr):
    s = 19000 + 10 * i
    shape = (n, k) if tr == "N" else (k, n)
    return U(s, *shape), U(s + 1, *shape), U(s + 2, n, n)


def tri_case_list():
    """(n, uplo, diag) for dtrtri and n for dgetri (on dgetrf's factors)."""
    cases = []
    for n in (1, 2, 5, 31, 64, 65, 129, 200):
        for uplo in "UL":
            for diag in "NU":
                cases.append((n, uplo, diag))
    return [(f"trtri{i:03d}", c) for i, c in enumerate(cases)]


def tri_input(i, n):
    A = U(21000 + 10 * i, n, n)
    A[np.arange(n), np.arange(n)] += 2.0 + n / 4.0
    return A


def getri_case_list():
    return [(f"getri{i:03d}", n) for i, n in enumerate((1, 2, 7, 31, 64, 65, 100, 129, 200))]


def getri_input(i, n):
    A = U(23000 + 10 * i, n, n)
    A[np.arange(n), np.arange(n)] += n / 4.0
    return A


def refine_case_list():
    """n for gecon / gerfs / geequ / laqge / gesvx (diagonally weighted uniform
    matrices, one column and one row badly scaled for the equilibration)."""
    return [(f"rfs{i:03d}", n) for i, n in enumerate((1, 2, 5, 31, 64, 65, 100))]


def refine_inputs(i, n):
    A = U(25000 + 10 * i, n, n)
    A[np.arange(n), np.arange(n)] += n / 8.0 + 0.5
    Ae = A.copy(order="F")
    Ae[:, 1 % n] *= 1.0e6
    Ae[0, :] *= 1.0e-5
    B = U(25000 + 10 * i + 1, n, 3)
    return A, Ae, B


def chol_case_list():
    """(n, uplo, kind): kind 'spd' (well conditioned) or 'notpd' (a negative
    pivot at n//2, so INFO = n//2 + 1 with the factor of the leading block)."""
    cases = []
    for n in (1, 2, 5, 31, 63, 64, 65, 100, 129, 200):
        for uplo in "LU":
            cases.append((n, uplo, "spd"))
    for n in (5, 64, 130):
        for uplo in "LU":
            cases.append((n, uplo, "notpd"))
    return [(f"chol{i:03d}", c) for i, c in enumerate(cases)]


def chol_input(i, n, kind):
    """Symmetric positive definite: G G^T / n + I with G splitmix uniform; the
    'notpd' kind sets A(n//2, n//2) = -1."""
    G = U(13000 + 10 * i, n, n)
    A = np.asfortranarray(G @ G.T / max(n, 1) + np.eye(n))
    if kind == "notpd":
        A[n // 2, n // 2] = -1.0
    return A


def chol_rhs(i, n):
    return U(13000 + 10 * i + 1, n, 3)


LARGE_N, LARGE_SEED = 8192, 20261203


def large_lu_input():
    """Config-2 input: n=8192, uniform[-1,1) + (n/4) I (splitmix seed LARGE_SEED)."""
    return oracle.shifted_square(LARGE_SEED, LARGE_N)


# ------------------------------------------------------------- generate --
def generate_small(R):
    out = {}
    for i, (name, (m, n, k, ta, tb, a, b)) in enumerate(gemm_case_list()):
        A, B, C = gemm_inputs(i, m, n, k, ta, tb)
        out[name] = R.dgemm(ta, tb, a, A, B, b, C.copy(order="F"))
    for i, (name, (m, n, side, uplo, ta, diag, alpha)) in enumerate(trsm_case_list()):
        A, B = trsm_inputs(i, m, n, side)
        out[name] = R.dtrsm(side, uplo, ta, diag, alpha, A, B.copy(order="F"))
    for i, (name, (m, n, kind)) in enumerate(lu_case_list()):
        LU = lu_input(i, m, n, kind)
        piv, info = R.dgetrf(LU)
        out[name + "_LU"], out[name + "_piv"] = LU, piv.astype(np.int32)
        out[name + "_info"] = np.array([info])
        if m == n:
            Bm = lu_rhs(i, n)
            for t in "NT":
                X, _ = R.dgetrs(t, LU, piv, Bm.copy(order="F"))
                out[name + f"_X{t}"] = X
    LU = singular_input()
    piv, info = R.dgetrf(LU)
    out["sing_LU"], out["sing_piv"], out["sing_info"] = LU, piv.astype(np.int32), np.array([info])
    for i, (name, (n, k, uplo, tr, a, b)) in enumerate(syrk_case_list()):
        A, C = syrk_inputs(i, n, k, tr)
        out[name] = R.dsyrk(uplo, tr, a, A, b, C.copy(order="F"))
    for i, (name, (m, n, side, uplo, ta, diag, alpha)) in enumerate(trmm_case_list()):
        A, B = trmm_inputs(i, m, n, side)
        out[name] = R.dtrmm(side, uplo, ta, diag, alpha, A, B.copy(order="F"))
    for i, (name, (m, n, side, uplo, a, b)) in enumerate(symm_case_list()):
        A, B, C = symm_inputs(i, m, n, side)
        out[name] = R.dsymm(side, uplo, a, A, B, b, C.copy(order="F"))
    for i, (name, (n, k, uplo, tr, a, b)) in enumerate(syr2k_case_list()):
        A, B, C = syr2k_inputs(i, n, k, tr)
        out[name] = R.dsyr2k(uplo, tr, a, A, B, b, C.copy(order="F"))
    for i, (name, (n, uplo, diag)) in enumerate(tri_case_list()):
        A = tri_input(i, n)
        R.dtrtri(uplo, diag, A)
        out[name] = A
    for i, (name, n) in enumerate(getri_case_list()):
        LU = getri_input(i, n)
        piv, info = R.dgetrf(LU)
        R.dgetri(LU, piv)
        out[name] = LU
    for i, (name, n) in enumerate(refine_case_list()):
        A, Ae, B = refine_inputs(i, n)
        LU = A.copy(order="F")
        piv, _ = R.dgetrf(LU)
        rc = [R.dgecon(nm, LU.copy(order="F"), oracle.Port().dlange("1" if nm != "I" else "I", A))[0]
              for nm in ("1", "I")]
        out[name + "_rcond"] = np.array(rc)
        for tr in "NT":
            X = B.copy(order="F")
            R.dgetrs(tr, LU.copy(order="F"), piv, X)
            X[0, :] += 1e-8                                   # start away from the solution
            ferr, berr = R.dgerfs(tr, A, LU.copy(order="F"), piv, B, X)
            out[name + f"_rfs{tr}_X"], out[name + f"_rfs{tr}_ferr"] = X, ferr
            out[name + f"_rfs{tr}_berr"] = berr
        r, c, rcnd, ccnd, amax, info = R.dgeequ(Ae.copy(order="F"))
        out[name + "_equ"] = np.concatenate([r, c, [rcnd, ccnd, amax, info]])
        for fact in "NE":
            for tr in "NT":
                Aw, Bw = Ae.copy(order="F"), B.copy(order="F")
                AF, Xw = np.zeros((n, n), order="F"), np.zeros((n, 3), order="F")
                pv = np.zeros(n, dtype=np.int32)
                info, eq, rcn, fe, be, g = R.dgesvx(fact, tr, Aw, AF, pv, "N", np.zeros(n),
                                                    np.zeros(n), Bw, Xw)
                k = name + f"_svx{fact}{tr}"
                out[k + "_X"], out[k + "_AF"], out[k + "_A"] = Xw, AF, Aw
                out[k + "_s"] = np.concatenate([[info, rcn, g], fe, be])
    # a singular system through gesvx: INFO, reciprocal pivot growth, rcond 0
    A = singular_input()
    n = A.shape[0]
    AF, X = np.zeros((n, n), order="F"), np.zeros((n, 1), order="F")
    info, eq, rcn, fe, be, g = R.dgesvx("N", "N", A, AF, np.zeros(n, dtype=np.int32), "N",
                                        np.zeros(n), np.zeros(n), U(7778, n, 1), X)
    out["svx_sing_s"] = np.array([info, rcn, g])
    for i, (name, (n, uplo, kind)) in enumerate(chol_case_list()):
        A = chol_input(i, n, kind)
        info = R.dpotrf(uplo, A)
        out[name + "_A"], out[name + "_info"] = A, np.array([info])
        if info == 0:
            X, _ = R.dpotrs(uplo, A, chol_rhs(i, n).copy(order="F"))
            out[name + "_X"] = X
    A, b = baby_problem()
    piv, info = R.dgesv(A, b)
    out["baby_LU"], out["baby_x"], out["baby_piv"] = A, b, piv.astype(np.int32)
    out["baby_info"] = np.array([info])
    return out


def generate_large(R):
    A = large_lu_input()
    piv, info = R.dgetrf(A)
    n = LARGE_N
    nonid = int(np.count_nonzero(piv != np.arange(1, n + 1)))
    return {"meta": np.array([n, LARGE_SEED, info, nonid], dtype=np.int64),
            "piv": piv.astype(np.int32),
            "diagU": np.ascontiguousarray(np.diag(A)),
            "colsum_LU": A.sum(axis=0)}


# Unshifted uniform[-1,1) matrices: LU with real row interchanges at sizes
# where the GPU's blocked summation order differs from the reference's, for
# pivot-vector parity at scale.  Stored per n: the reference's pivots and
# INFO, diag(U) of its factors, and the relative gap between the two largest
# |candidates| of every pivot search (from the oracle restatement, which must
# give the reference's pivots bit for bit on the same input).
PIVOT_CASES = ((2048, 777), (4096, 778))


def generate_pivots(R):
    P = oracle.Port()
    out = {}
    for n, seed in PIVOT_CASES:
        A = oracle.splitmix_uniform(seed, n, n)
        Ar = A.copy(order="F")
        piv, info = R.dgetrf(Ar)
        pp, pinfo, gap = P.dgetrf_gaps(A.copy(order="F"))
        assert info == pinfo and np.array_equal(piv, pp), "restatement differs from the reference"
        out[f"n{n}_meta"] = np.array([n, seed, info], dtype=np.int64)
        out[f"n{n}_piv"] = piv.astype(np.int32)
        out[f"n{n}_gap"] = gap
        out[f"n{n}_diagU"] = np.ascontiguousarray(np.diag(Ar))
        print(f"n={n}: {int(np.count_nonzero(piv != np.arange(1, n + 1)))} interchanges, "
              f"smallest gap {gap.min():.3e}")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--large", action="store_true")
    ap.add_argument("--pivots", action="store_true",
                    help="+ the unshifted n=2048/4096 pivot fixtures (a few minutes)")
    ap.add_argument("--no-small", action="store_true")
    args = ap.parse_args()
    oracle.build(with_ref=True)
    R = oracle.Reference()
    if not args.no_small:
        small = generate_small(R)
        path = os.path.join(HERE, "reference_small.npz")
        np.savez_compressed(path, **small)
        print(f"wrote {path} ({os.path.getsize(path)} bytes, {len(small)} arrays)")
    if args.pivots:
        piv = generate_pivots(R)
        p3 = os.path.join(HERE, "reference_lu_unshifted.npz")
        np.savez_compressed(p3, **piv)
        print(f"wrote {p3} ({os.path.getsize(p3)} bytes)")
    if args.large:
        big = generate_large(R)
        p2 = os.path.join(HERE, "reference_lu8192.npz")
        np.savez_compressed(p2, **big)
        print(f"wrote {p2}: meta(n, seed, info, non-identity pivots)={big['meta'].tolist()}")


if __name__ == "__main__":
    main()
