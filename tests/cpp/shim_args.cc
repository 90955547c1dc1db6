// Compiled by tests/test_cpp_shim.py against the FLENS headers, the C++
// drop-in header and tests/cpp/abi_recorder.c: each FLENS call below prints
// the Fortran-ABI call it became (see the expected lines in the test).
#include <flens_gb300/flens_gb300.hpp>

#include <cstdio>

using namespace flens;

typedef GeMatrix<FullStorage<double, ColMajor> > CMatrix;
typedef GeMatrix<FullStorage<double, RowMajor> > RMatrix;

int main()
{
    // column-major, 3 x 5 times 5 x 2
    CMatrix A(3, 5), B(5, 2), C(3, 2);
    A = 1; B = 1; C = 0;
    std::printf("# gemm col\n");
    C = A * B;
    // row-major storage of the same shapes: FLENS calls cxxblas with RowMajor
    RMatrix Ar(3, 5), Br(5, 2), Cr(3, 2);
    Ar = 1; Br = 1; Cr = 0;
    std::printf("# gemm row\n");
    Cr = Ar * Br;

    CMatrix K(4, 6), S(4, 4);
    K = 1; S = 0;
    std::printf("# syrk col\n");
    blas::rk(NoTrans, 1.0, K, 0.0, S.upper().symmetric());
    RMatrix Kr(4, 6), Sr(4, 4);
    Kr = 1; Sr = 0;
    std::printf("# syrk row\n");
    blas::rk(NoTrans, 1.0, Kr, 0.0, Sr.upper().symmetric());
    std::printf("# syr2k row\n");
    blas::r2k(NoTrans, 1.0, Kr, Kr, 0.0, Sr.upper().symmetric());

    CMatrix T(3, 3), E(3, 7);
    T = 1; E = 1;
    std::printf("# trmm col\n");
    blas::mm(Left, NoTrans, 2.0, T.upper(), E);
    RMatrix Tr(3, 3), Er(3, 7);
    Tr = 1; Er = 1;
    std::printf("# trmm row\n");
    blas::mm(Left, NoTrans, 2.0, Tr.upper(), Er);
    std::printf("# symm row\n");
    RMatrix Fr(3, 7);
    Fr = 0;
    blas::mm(Left, 1.0, Tr.upper().symmetric(), Er, 0.0, Fr);
    std::printf("# trsm row\n");
    blas::sm(Left, NoTrans, 1.0, Tr.lowerUnit(), Er);

    std::printf("# lapack\n");
    CMatrix P(4, 4), X(4, 2), R(4, 2), AF(4, 4);
    DenseVector<Array<int> > piv(4), iw(4);
    DenseVector<Array<double> > fErr(2), bErr(2), r(4), c(4), w3(12), w4(16);
    P = 1; X = 0; R = 1;
    lapack::trf(P, piv);
    lapack::trs(NoTrans, P, piv, R);
    lapack::potrf(P.lower().symmetric());
    lapack::potrs(P.lower().symmetric(), R);
    lapack::tri(P.upperUnit());
    lapack::tri(P, piv, w4);
    lapack::rfs(Trans, P, P, piv, R, X, fErr, bErr, w3, iw);
    double rc = -1, rcnd = 0, ccnd = 0, amax = 0;
    lapack::con(lapack::InfinityNorm, P, 3.0, rc, w4, iw);
    lapack::equ(P, r, c, rcnd, ccnd, amax);
    lapack::laq(P, r, c, rcnd, ccnd, amax);
    lapack::svx(lapack::SVX::Equilibrate, NoTrans, P, AF, piv, lapack::SVX::None, r, c, R, X, rc,
                fErr, bErr, w4, iw);
    std::printf("# done rcond=%g\n", rc);
    return 0;
}
