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
REF = "/root/reference"


@pytest.fixture(scope="module")
def shim_binary(tmp_path_factory):
    if not os.path.isdir(REF):
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
