"""The C++ drop-in header routes FLENS's own entry points to the library.

Builds tests/cpp/shim_routing.cc against the FLENS headers (only where they
are present) and include/flens_gb300/flens_gb300.hpp, linked with
libflens_gb300.so.  Without a GPU every routed call must fail loudly with the
library's no-device error instead of computing on the CPU -- which proves that
blas::mm, sm, rk, r2k and lapack::trf, potrf, potrs, tri, rfs, con, equ, svx no
longer run the reference's generic code.
With a GPU the same program must print the reference's answers.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ref_dir():
    import oracle
    return oracle.REFERENCE_SRC


REF = _ref_dir()


@pytest.fixture(scope="module")
def shim_binary(tmp_path_factory):
    if not REF or not os.path.isdir(REF):
        pytest.skip("FLENS headers not present on this machine")
    import flens_gb300
    flens_gb300.lib()
    out = str(tmp_path_factory.mktemp("shim") / "shim_routing")
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I" + REF, "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_routing.cc"), "-o", out,
           "-L" + os.path.join(ROOT, "flens_gb300"), "-lflens_gb300",
           "-Wl,-rpath," + os.path.join(ROOT, "flens_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_flens_calls_reach_the_library_without_gpu(shim_binary):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([shim_binary], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # generic FLENS would have computed C(1,1) = 4 and trf info = 0
    assert "dgemm_ failed (-1003)" in r.stderr
    assert "dtrsm_ failed (-1003)" in r.stderr
    assert "trf info=-1003" in r.stdout
    for f in ("dsyrk_", "dsyr2k_", "dsymm_", "dtrmm_", "dpotrs_"):
        assert f + " failed (-1003)" in r.stderr, f
    for f in ("potrf", "trtri", "getri", "equ"):
        assert f + " info=-1003" in r.stdout, f
    for f in ("dgerfs_", "dgecon_"):
        assert f + " failed (-1003)" in r.stderr, f
    # the expert driver fails in its workspace request: any library error
    assert "dgesvx_ failed (-100" in r.stderr and "svx info=-100" in r.stdout


# The Fortran-ABI calls FLENS's own entry points become (tests/cpp/shim_args.cc
# against the argument recorder tests/cpp/abi_recorder.c).  Row-major FLENS
# storage is the transposed column-major problem: gemm swaps the operands,
# syrk/syr2k take the other triangle and the transposed operand, trmm, symm
# and trsm move to the other side and triangle.
EXPECTED_ARGS = """\
# gemm col
dgemm_ N N m=3 n=2 k=5 lda=3 ldb=5 ldc=3 alpha=1 beta=0
# gemm row
dgemm_ N N m=2 n=3 k=5 lda=2 ldb=5 ldc=2 alpha=1 beta=0
# syrk col
dsyrk_ U N n=4 k=6 lda=4 ldc=4
# syrk row
dsyrk_ L T n=4 k=6 lda=6 ldc=4
# syr2k row
dsyr2k_ L T n=4 k=6 lda=6 ldb=6 ldc=4
# trmm col
dtrmm_ L U N N m=3 n=7 lda=3 ldb=3
# trmm row
dtrmm_ R L N N m=7 n=3 lda=3 ldb=7
# symm row
dsymm_ R L m=7 n=3 lda=3 ldb=7 ldc=7
# trsm row
dtrsm_ R U N U m=7 n=3 lda=3 ldb=7
# lapack
dgetrf_ m=4 n=4 lda=4
dgetrs_ N n=4 nrhs=2 lda=4 ldb=4
dpotrf_ L n=4 lda=4
dpotrs_ L n=4 nrhs=2 lda=4 ldb=4
dtrtri_ U U n=4 lda=4
dgetri_ n=4 lda=4 lwork=4
dgerfs_ T n=4 nrhs=2 lda=4 ldaf=4 ldb=4 ldx=4
dgecon_ I n=4 lda=4 anorm=3
dgeequ_ m=4 n=4 lda=4
dlaqge_ m=4 n=4 lda=4
dgesvx_ E N equed=N n=4 nrhs=2 lda=4 ldaf=4 ldb=4 ldx=4
# done rcond=0.5
"""


def test_flens_calls_map_to_the_fortran_abi(tmp_path):
    if not REF or not os.path.isdir(REF):
        pytest.skip("FLENS headers not present on this machine")
    rec = str(tmp_path / "abi_recorder.o")
    r = subprocess.run(["gcc", "-c", "-O1", os.path.join(ROOT, "tests", "cpp", "abi_recorder.c"),
                        "-o", rec], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = str(tmp_path / "shim_args")
    r = subprocess.run(["g++", "-std=c++11", "-O1", "-w", "-I" + REF, "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "shim_args.cc"), rec, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout == EXPECTED_ARGS, r.stdout
