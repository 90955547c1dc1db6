// Compiled by tests/test_cpp_shim.py against the FLENS headers and
// include/flens_gb300/flens_gb300.hpp.  Prints one line per routed call so the
// test can tell whether FLENS's own entry points reached libflens_gb300.so.
#include <flens_gb300/flens_gb300.hpp>

#include <cstdio>

using namespace flens;

typedef GeMatrix<FullStorage<double, ColMajor> > RealGeMatrix;
typedef DenseVector<Array<int> > IndexVector;

int main()
{
    const int n = 4;
    RealGeMatrix A(n, n), B(n, n), C(n, n);
    IndexVector piv(n);
    // the system of flens/examples/lapack-gesv.cc
    A = 2, 3, -1, 0,
        -6, -5, 0, 2,
        2, -5, 6, -6,
        4, 6, 2, -3;
    B = 1;
    C = 0;
    C = 2.0*A*B;                                       // -> blas::mm -> cxxblas::gemm
    std::printf("mm C(1,1)=%g\n", C(1, 1));
    blas::sm(Left, NoTrans, 1.0, A.lowerUnit(), B);    // -> cxxblas::trsm
    std::printf("sm B(2,1)=%g\n", B(2, 1));
    const int info = lapack::trf(A, piv);              // -> generic::trf_impl -> dgetrf_
    std::printf("trf info=%d piv=%d,%d,%d,%d\n", info, piv(1), piv(2), piv(3), piv(4));

    // the rest of level 3
    RealGeMatrix D(n, n), E(n, n);
    D = 1;
    E = 0;
    blas::rk(NoTrans, 1.0, D, 0.0, E.upper().symmetric());          // -> cxxblas::syrk
    blas::r2k(NoTrans, 1.0, D, D, 0.0, E.upper().symmetric());      // -> cxxblas::syr2k
    blas::mm(Left, 1.0, D.upper().symmetric(), D, 0.0, E);          // -> cxxblas::symm
    blas::mm(Left, NoTrans, 1.0, D.upper(), E);                      // -> cxxblas::trmm
    std::printf("level3 E(1,1)=%g\n", E(1, 1));

    // Cholesky and the inverses
    RealGeMatrix S(n, n);
    S = 4, 1, 0, 0,
        1, 4, 1, 0,
        0, 1, 4, 1,
        0, 0, 1, 4;
    const int pinfo = lapack::potrf(S.upper().symmetric());         // -> generic::potrf_impl
    std::printf("potrf info=%d\n", pinfo);
    lapack::potrs(S.upper().symmetric(), D);                         // -> generic::potrs_impl
    const int tinfo = lapack::tri(S.upper());                        // -> (tr) generic::tri_impl
    std::printf("trtri info=%d\n", tinfo);
    DenseVector<Array<double> > work(n);
    const int ginfo = lapack::tri(A, piv, work);                     // -> (ge) generic::tri_impl
    std::printf("getri info=%d\n", ginfo);

    // refinement, condition, equilibration, expert driver
    RealGeMatrix X(n, n);
    X = 0;
    DenseVector<Array<double> > fErr(n), bErr(n), r(n), c(n), w3(3 * n), w4(4 * n);
    DenseVector<Array<int> > iw(n);
    lapack::rfs(NoTrans, S, S, piv, D, X, fErr, bErr, w3, iw);       // -> generic::rfs_impl
    double rcond = -1;
    lapack::con(lapack::OneNorm, S, 1.0, rcond, w4, iw);             // -> generic::con_impl
    std::printf("con rcond=%g\n", rcond);
    double rowCond = -1, colCond = -1, amax = -1;
    const int einfo = lapack::equ(S, r, c, rowCond, colCond, amax); // -> generic::equ_impl
    std::printf("equ info=%d\n", einfo);
    RealGeMatrix AF(n, n);
    IndexVector piv2(n);
    const int sinfo = lapack::svx(lapack::SVX::NotFactored, NoTrans, S, AF, piv2,
                                  lapack::SVX::None, r, c, D, X, rcond, fErr, bErr, w4, iw);
    std::printf("svx info=%d\n", sinfo);
    std::printf("last_error=%s\n", flens_gb300_last_error());
    return 0;
}
