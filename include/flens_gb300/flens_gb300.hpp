/*
 * flens_gb300.hpp -- route FLENS's dense GEMM / TRSM / LU to the GB300 library.
 *
 * Include this header INSTEAD OF <flens/flens.cxx> (it includes FLENS itself):
 *
 *     #include <flens_gb300/flens_gb300.hpp>     // was: #include <flens/flens.cxx>
 *     ...   link with -lflens_gb300
 *
 * It plugs into the two places FLENS already provides for a faster backend:
 *
 *  - cxxblas level 3: like the cblas overloads FLENS adds under HAVE_CBLAS
 *    (cxxblas/level3/gemm.tcc:218-240, cxxblas/level3/trsm.tcc:107-126), more
 *    specialised overloads of cxxblas::gemm, trsm, syrk, syr2k, trmm and symm
 *    for double with an integral index forward to dgemm_, dtrsm_, dsyrk_,
 *    dsyr2k_, dtrmm_ and dsymm_.  flens::blas::mm, sm, rk, r2k
 *    (flens/blas/level3/mm.tcc:463-472, sm.tcc:61-67, ...), the operator form
 *    C = beta*C + alpha*A*B, and every level-3 call FLENS-LAPACK makes reach
 *    them.
 *  - FLENS-LAPACK's generic implementations: more specialised overloads of
 *    flens::lapack::generic::trf_impl (flens/lapack/ge/trf.tcc:61), trs_impl
 *    (flens/lapack/ge/trs.tcc:61), potrf_impl (flens/lapack/po/potrf.tcc:61),
 *    potrs_impl (flens/lapack/po/potrs.tcc:61), the two tri_impl
 *    (flens/lapack/ge/tri.tcc:64, flens/lapack/tr/tri.tcc:64), rfs_impl
 *    (flens/lapack/ge/rfs.tcc:63), con_impl (flens/lapack/ge/cond.tcc:62),
 *    equ_impl (flens/lapack/ge/equ.tcc:62), laq_impl
 *    (flens/lapack/la/laq.tcc:59) and svx_impl (flens/lapack/ge/svx.tcc:60)
 *    for column-major double matrices with int pivots forward to dgetrf_,
 *    dgetrs_, dpotrf_, dpotrs_, dgetri_, dtrtri_, dgerfs_, dgecon_, dgeequ_,
 *    dlaqge_ and dgesvx_, so lapack::trf, trs, sv, potrf, potrs, posv, tri,
 *    rfs, con, equ and svx run on the GPU.  Other element types, index types
 *    and storage orders keep the reference's generic code.
 *
 * The overloads must be declared between flens.h and flens.tcc so that the
 * qualified calls inside the FLENS templates see them; hence the include
 * order below.  Memory may be host (copied to the GPU per call) or device /
 * managed (used in place).
 */
#ifndef FLENS_GB300_FLENS_GB300_HPP
#define FLENS_GB300_FLENS_GB300_HPP 1

#ifdef FLENS_FLENS_CXX
#error "include <flens_gb300/flens_gb300.hpp> instead of (not after) <flens/flens.cxx>"
#endif

#include <cstdio>
#include <type_traits>
#include <vector>

#include <flens/flens.h>
#include <flens_gb300.h>

namespace flens_gb300 { namespace detail {

inline char trans_char(cxxblas::Transpose t)
{
    return (static_cast<int>(t) & static_cast<int>(cxxblas::Trans)) ? 'T' : 'N';
}

template <typename IndexType>
struct IsIndex
{
    static const bool value = std::is_integral<IndexType>::value;
};

template <typename S>
struct IsDoubleColMajorFull : std::false_type {};

template <typename I, typename A>
struct IsDoubleColMajorFull<flens::FullStorage<double, cxxblas::ColMajor, I, A> >
    : std::true_type {};

template <typename I, typename A>
struct IsDoubleColMajorFull<flens::FullStorageView<double, cxxblas::ColMajor, I, A> >
    : std::true_type {};

template <typename I, typename A>
struct IsDoubleColMajorFull<flens::ConstFullStorageView<double, cxxblas::ColMajor, I, A> >
    : std::true_type {};

// element i (0-based, logical order) of a FLENS vector, copied out / in
template <typename T, typename V>
inline std::vector<T> to_vec(const flens::DenseVector<V> &x)
{
    std::vector<T> v(x.length() > 0 ? std::size_t(x.length()) : 1);
    for (int i = 0; i < int(x.length()); ++i) v[i] = T(x(x.firstIndex() + i));
    return v;
}

template <typename T, typename V>
inline void from_vec(const std::vector<T> &v, flens::DenseVector<V> &x)
{
    for (int i = 0; i < int(x.length()); ++i) x(x.firstIndex() + i) = v[i];
}

}  // namespace detail
}  // namespace flens_gb300

namespace cxxblas {

//-- gemm: double, any integral index -> dgemm_ (column-major)
template <typename IndexType>
typename std::enable_if<flens_gb300::detail::IsIndex<IndexType>::value, void>::type
gemm(StorageOrder order, Transpose transA, Transpose transB,
     IndexType m, IndexType n, IndexType k,
     double alpha, const double *A, IndexType ldA,
     const double *B, IndexType ldB,
     double beta, double *C, IndexType ldC)
{
    if (order == RowMajor) {
        // C^T = op(B)^T op(A)^T in column-major terms (cxxblas/level3/gemm.tcc:57-64)
        gemm(ColMajor, transB, transA, n, m, k, alpha, B, ldB, A, ldA, beta, C, ldC);
        return;
    }
    const char ta = flens_gb300::detail::trans_char(transA);
    const char tb = flens_gb300::detail::trans_char(transB);
    const int M = int(m), N = int(n), K = int(k);
    const int LDA = int(ldA), LDB = int(ldB), LDC = int(ldC);
    dgemm_(&ta, &tb, &M, &N, &K, &alpha, A, &LDA, B, &LDB, &beta, C, &LDC);
}

//-- trsm: double, any integral index -> dtrsm_ (column-major)
template <typename IndexType>
typename std::enable_if<flens_gb300::detail::IsIndex<IndexType>::value, void>::type
trsm(StorageOrder order, Side side, StorageUpLo upLo, Transpose transA, Diag diag,
     IndexType m, IndexType n, double alpha,
     const double *A, IndexType ldA, double *B, IndexType ldB)
{
    if (order == RowMajor) {
        // row-major B is column-major B^T (cxxblas/level3/trsm.tcc:48-52)
        trsm(ColMajor, side == Left ? Right : Left, upLo == Upper ? Lower : Upper, transA,
             diag, n, m, alpha, A, ldA, B, ldB);
        return;
    }
    const char s = static_cast<char>(side), u = static_cast<char>(upLo);
    const char t = flens_gb300::detail::trans_char(transA), d = static_cast<char>(diag);
    const int M = int(m), N = int(n), LDA = int(ldA), LDB = int(ldB);
    dtrsm_(&s, &u, &t, &d, &M, &N, &alpha, A, &LDA, B, &LDB);
}

//-- syrk: double, any integral index -> dsyrk_ (column-major)
template <typename IndexType>
typename std::enable_if<flens_gb300::detail::IsIndex<IndexType>::value, void>::type
syrk(StorageOrder order, StorageUpLo upLo, Transpose trans, IndexType n, IndexType k,
     double alpha, const double *A, IndexType ldA, double beta, double *C, IndexType ldC)
{
    if (order == RowMajor) {
        // the row-major triangle is the column-major opposite one, op(A)
        // flips (cxxblas/level3/syrk.tcc:51-56)
        syrk(ColMajor, upLo == Upper ? Lower : Upper, Transpose(trans ^ Trans), n, k, alpha, A, ldA,
             beta, C, ldC);
        return;
    }
    const char u = static_cast<char>(upLo), t = flens_gb300::detail::trans_char(trans);
    const int N = int(n), K = int(k), LDA = int(ldA), LDC = int(ldC);
    dsyrk_(&u, &t, &N, &K, &alpha, A, &LDA, &beta, C, &LDC);
}

//-- syr2k: double, any integral index -> dsyr2k_ (column-major)
template <typename IndexType>
typename std::enable_if<flens_gb300::detail::IsIndex<IndexType>::value, void>::type
syr2k(StorageOrder order, StorageUpLo upLo, Transpose trans, IndexType n, IndexType k,
      double alpha, const double *A, IndexType ldA, const double *B, IndexType ldB,
      double beta, double *C, IndexType ldC)
{
    if (order == RowMajor) {
        // (cxxblas/level3/syr2k.tcc:52-57)
        syr2k(ColMajor, upLo == Upper ? Lower : Upper, Transpose(trans ^ Trans), n, k, alpha, A, ldA,
              B, ldB, beta, C, ldC);
        return;
    }
    const char u = static_cast<char>(upLo), t = flens_gb300::detail::trans_char(trans);
    const int N = int(n), K = int(k), LDA = int(ldA), LDB = int(ldB), LDC = int(ldC);
    dsyr2k_(&u, &t, &N, &K, &alpha, A, &LDA, B, &LDB, &beta, C, &LDC);
}

//-- trmm: double, any integral index -> dtrmm_ (column-major)
template <typename IndexType>
typename std::enable_if<flens_gb300::detail::IsIndex<IndexType>::value, void>::type
trmm(StorageOrder order, Side side, StorageUpLo upLo, Transpose transA, Diag diag,
     IndexType m, IndexType n, double alpha, const double *A, IndexType ldA,
     double *B, IndexType ldB)
{
    if (order == RowMajor) {
        // row-major B is column-major B^T: the other side, the other
        // triangle, m and n swapped (cxxblas/level3/trmm.tcc:49-54)
        trmm(ColMajor, side == Left ? Right : Left, upLo == Upper ? Lower : Upper, transA, diag, n, m,
             alpha, A, ldA, B, ldB);
        return;
    }
    const char sd = static_cast<char>(side), u = static_cast<char>(upLo);
    const char t = flens_gb300::detail::trans_char(transA), d = static_cast<char>(diag);
    const int M = int(m), N = int(n), LDA = int(ldA), LDB = int(ldB);
    dtrmm_(&sd, &u, &t, &d, &M, &N, &alpha, A, &LDA, B, &LDB);
}

//-- symm: double, any integral index -> dsymm_ (column-major)
template <typename IndexType>
typename std::enable_if<flens_gb300::detail::IsIndex<IndexType>::value, void>::type
symm(StorageOrder order, Side side, StorageUpLo upLo, IndexType m, IndexType n,
     double alpha, const double *A, IndexType ldA, const double *B, IndexType ldB,
     double beta, double *C, IndexType ldC)
{
    if (order == RowMajor) {
        // (cxxblas/level3/symm.tcc:51-58)
        symm(ColMajor, side == Left ? Right : Left, upLo == Upper ? Lower : Upper, n, m, alpha, A, ldA,
             B, ldB, beta, C, ldC);
        return;
    }
    const char sd = static_cast<char>(side), u = static_cast<char>(upLo);
    const int M = int(m), N = int(n), LDA = int(ldA), LDB = int(ldB), LDC = int(ldC);
    dsymm_(&sd, &u, &M, &N, &alpha, A, &LDA, B, &LDB, &beta, C, &LDC);
}

}  // namespace cxxblas

namespace flens { namespace lapack { namespace generic {

//-- trf for column-major double with int pivots -> dgetrf_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename VP>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value
        && std::is_same<typename DenseVector<VP>::ElementType, int>::value,
    typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType>::type
trf_impl(GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A, DenseVector<VP> &piv)
{
    typedef typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType IndexType;
    const int m = int(A.numRows()), n = int(A.numCols());
    const int ld = int(A.leadingDimension() > 0 ? A.leadingDimension() : 1);
    const int mn = m < n ? m : n;
    int info = 0;
    if (m == 0 || n == 0) return IndexType(0);
    if (piv.stride() == 1) {
        dgetrf_(&m, &n, A.data(), &ld, piv.data(), &info);
    } else {
        std::vector<int> p(mn);
        dgetrf_(&m, &n, A.data(), &ld, p.data(), &info);
        for (int i = 0; i < mn; ++i) piv(piv.firstIndex() + i * (piv.inc() > 0 ? 1 : -1)) = p[i];
    }
    return IndexType(info);
}

//-- trs for column-major double with int pivots -> dgetrs_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FSA,
          typename IA, typename AA,
          template <typename, cxxblas::StorageOrder, typename, typename> class FSB,
          typename IB, typename AB, typename VP>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FSA<double, cxxblas::ColMajor, IA, AA> >::value
        && flens_gb300::detail::IsDoubleColMajorFull<FSB<double, cxxblas::ColMajor, IB, AB> >::value
        && std::is_same<typename DenseVector<VP>::ElementType, int>::value,
    void>::type
trs_impl(Transpose trans, const GeMatrix<FSA<double, cxxblas::ColMajor, IA, AA> > &A,
         const DenseVector<VP> &piv, GeMatrix<FSB<double, cxxblas::ColMajor, IB, AB> > &B)
{
    const int n = int(A.numCols()), nrhs = int(B.numCols());
    if (n == 0 || nrhs == 0) return;
    const int lda = int(A.leadingDimension()), ldb = int(B.leadingDimension());
    const char t = flens_gb300::detail::trans_char(trans);
    int info = 0;
    if (piv.stride() == 1) {
        dgetrs_(&t, &n, &nrhs, A.data(), &lda, piv.data(), B.data(), &ldb, &info);
    } else {
        std::vector<int> p(n);
        for (int i = 0; i < n; ++i) p[i] = piv(piv.firstIndex() + i * (piv.inc() > 0 ? 1 : -1));
        dgetrs_(&t, &n, &nrhs, A.data(), &lda, p.data(), B.data(), &ldb, &info);
    }
}

//-- potrf for column-major double -> dpotrf_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value,
    typename SyMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType>::type
potrf_impl(SyMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A)
{
    typedef typename SyMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType IndexType;
    const int n = int(A.dim());
    if (n == 0) return IndexType(0);
    const int ld = int(A.leadingDimension());
    const char u = static_cast<char>(A.upLo());
    int info = 0;
    dpotrf_(&u, &n, A.data(), &ld, &info);
    return IndexType(info);
}

//-- potrs for column-major double -> dpotrs_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FSA,
          typename IA, typename AA,
          template <typename, cxxblas::StorageOrder, typename, typename> class FSB,
          typename IB, typename AB>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FSA<double, cxxblas::ColMajor, IA, AA> >::value
        && flens_gb300::detail::IsDoubleColMajorFull<FSB<double, cxxblas::ColMajor, IB, AB> >::value,
    void>::type
potrs_impl(const SyMatrix<FSA<double, cxxblas::ColMajor, IA, AA> > &A,
           GeMatrix<FSB<double, cxxblas::ColMajor, IB, AB> > &B)
{
    const int n = int(A.dim()), nrhs = int(B.numCols());
    if (n == 0 || nrhs == 0) return;
    const int lda = int(A.leadingDimension()), ldb = int(B.leadingDimension());
    const char u = static_cast<char>(A.upLo());
    int info = 0;
    dpotrs_(&u, &n, &nrhs, A.data(), &lda, B.data(), &ldb, &info);
    // potrs has no INFO to return: report a library failure (a CUDA error,
    // no device) the way the BLAS entry points do
    if (info <= -1000)
        std::fprintf(stderr, "[flens_gb300] dpotrs_ failed (%d): %s\n", info, flens_gb300_last_error());
}

//-- (ge)tri for column-major double with int pivots -> dgetri_ (the
//   library keeps its own device workspace; `work` is not needed)
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename VP, typename VWORK>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value
        && std::is_same<typename DenseVector<VP>::ElementType, int>::value,
    typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType>::type
tri_impl(GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A, const DenseVector<VP> &piv,
         DenseVector<VWORK> &)
{
    typedef typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType IndexType;
    const int n = int(A.numRows());
    if (n == 0) return IndexType(0);
    const int ld = int(A.leadingDimension());
    std::vector<int> p(n);
    for (int i = 0; i < n; ++i) p[i] = piv(piv.firstIndex() + i * (piv.inc() > 0 ? 1 : -1));
    std::vector<double> work(n);
    const int lwork = n;
    int info = 0;
    dgetri_(&n, A.data(), &ld, p.data(), work.data(), &lwork, &info);
    return IndexType(info);
}

//-- (tr)tri for column-major double -> dtrtri_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value,
    typename TrMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType>::type
tri_impl(TrMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A)
{
    typedef typename TrMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType IndexType;
    const int n = int(A.dim());
    if (n == 0) return IndexType(0);
    const int ld = int(A.leadingDimension());
    const char u = static_cast<char>(A.upLo()), d = static_cast<char>(A.diag());
    int info = 0;
    dtrtri_(&u, &d, &n, A.data(), &ld, &info);
    return IndexType(info);
}

//-- rfs (refinement and error bounds) -> dgerfs_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename MAF, typename VPIV, typename MB, typename MX,
          typename VFERR, typename VBERR, typename VWORK, typename VIWORK>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value
        && flens_gb300::detail::IsDoubleColMajorFull<MAF>::value
        && flens_gb300::detail::IsDoubleColMajorFull<MB>::value
        && flens_gb300::detail::IsDoubleColMajorFull<MX>::value
        && std::is_same<typename DenseVector<VPIV>::ElementType, int>::value,
    void>::type
rfs_impl(Transpose trans, const GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A,
         const GeMatrix<MAF> &AF, const DenseVector<VPIV> &piv, const GeMatrix<MB> &B,
         GeMatrix<MX> &X, DenseVector<VFERR> &fErr, DenseVector<VBERR> &bErr,
         DenseVector<VWORK> &, DenseVector<VIWORK> &)
{
    const int n = int(A.numRows()), nrhs = int(B.numCols());
    if (n == 0 || nrhs == 0) return;
    const int lda = int(A.leadingDimension()), ldaf = int(AF.leadingDimension());
    const int ldb = int(B.leadingDimension()), ldx = int(X.leadingDimension());
    const char t = flens_gb300::detail::trans_char(trans);
    std::vector<int> p = flens_gb300::detail::to_vec<int>(piv), iwork(n);
    std::vector<double> fe(nrhs), be(nrhs), work(3 * std::size_t(n));
    int info = 0;
    dgerfs_(&t, &n, &nrhs, A.data(), &lda, AF.data(), &ldaf, p.data(), B.data(), &ldb, X.data(),
            &ldx, fe.data(), be.data(), work.data(), iwork.data(), &info);
    if (info <= -1000)
        std::fprintf(stderr, "[flens_gb300] dgerfs_ failed (%d): %s\n", info, flens_gb300_last_error());
    flens_gb300::detail::from_vec(fe, fErr);
    flens_gb300::detail::from_vec(be, bErr);
}

//-- con (condition estimate from the LU factors) -> dgecon_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename NORMA, typename RCOND, typename VWORK,
          typename VIWORK>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value,
    void>::type
con_impl(Norm norm, const GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A,
         const NORMA &normA, RCOND &rCond, DenseVector<VWORK> &, DenseVector<VIWORK> &)
{
    const int n = int(A.numRows());
    const int lda = int(A.leadingDimension() > 0 ? A.leadingDimension() : 1);
    const char nm = static_cast<char>(norm);
    const double anorm = double(normA);
    double rc = 0.0;
    std::vector<double> work(4 * std::size_t(n > 0 ? n : 1));
    std::vector<int> iwork(n > 0 ? n : 1);
    int info = 0;
    dgecon_(&nm, &n, A.data(), &lda, &anorm, &rc, work.data(), iwork.data(), &info);
    if (info <= -1000)
        std::fprintf(stderr, "[flens_gb300] dgecon_ failed (%d): %s\n", info, flens_gb300_last_error());
    rCond = rc;
}

//-- equ (row and column scalings) -> dgeequ_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename VR, typename VC, typename ROWCOND,
          typename COLCOND, typename AMAX>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value,
    typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType>::type
equ_impl(const GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A, DenseVector<VR> &r,
         DenseVector<VC> &c, ROWCOND &rowCond, COLCOND &colCond, AMAX &amax)
{
    typedef typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType IndexType;
    const int m = int(A.numRows()), n = int(A.numCols());
    const int lda = int(A.leadingDimension() > 0 ? A.leadingDimension() : 1);
    std::vector<double> rv(m > 0 ? m : 1), cv(n > 0 ? n : 1);
    double rc = 0.0, cc = 0.0, am = 0.0;
    int info = 0;
    dgeequ_(&m, &n, A.data(), &lda, rv.data(), cv.data(), &rc, &cc, &am, &info);
    flens_gb300::detail::from_vec(rv, r);
    flens_gb300::detail::from_vec(cv, c);
    rowCond = rc;
    colCond = cc;
    amax = am;
    return IndexType(info);
}

//-- laq (apply the scalings when worthwhile) -> dlaqge_
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename VR, typename VC, typename ROWCOND,
          typename COLCOND, typename AMAX>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value,
    LAQ::Equilibration>::type
laq_impl(GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A, const DenseVector<VR> &r,
         const DenseVector<VC> &c, const ROWCOND &rowCond, const COLCOND &colCond,
         const AMAX &amax)
{
    const int m = int(A.numRows()), n = int(A.numCols());
    const int lda = int(A.leadingDimension() > 0 ? A.leadingDimension() : 1);
    const std::vector<double> rv = flens_gb300::detail::to_vec<double>(r);
    const std::vector<double> cv = flens_gb300::detail::to_vec<double>(c);
    const double rc = double(rowCond), cc = double(colCond), am = double(amax);
    char equed = 'N';
    dlaqge_(&m, &n, A.data(), &lda, rv.data(), cv.data(), &rc, &cc, &am, &equed);
    return LAQ::Equilibration(equed);
}

//-- svx (expert driver) -> dgesvx_.  EQUED is taken by value, as in the
//   reference's interface, so the scaling applied is not reported back
//   through it; work(1) receives the reciprocal pivot growth.
template <template <typename, cxxblas::StorageOrder, typename, typename> class FS,
          typename I, typename Alloc, typename MAF, typename VPIV, typename VR, typename VC,
          typename MB, typename MX, typename RCOND, typename FERR, typename BERR,
          typename VWORK, typename VIWORK>
typename std::enable_if<
    flens_gb300::detail::IsDoubleColMajorFull<FS<double, cxxblas::ColMajor, I, Alloc> >::value
        && flens_gb300::detail::IsDoubleColMajorFull<MAF>::value
        && flens_gb300::detail::IsDoubleColMajorFull<MB>::value
        && flens_gb300::detail::IsDoubleColMajorFull<MX>::value
        && std::is_same<typename DenseVector<VPIV>::ElementType, int>::value,
    typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType>::type
svx_impl(SVX::Fact fact, Transpose trans, GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> > &A,
         GeMatrix<MAF> &AF, DenseVector<VPIV> &piv, SVX::Equilibration equed,
         DenseVector<VR> &r, DenseVector<VC> &c, GeMatrix<MB> &B, GeMatrix<MX> &X,
         RCOND &rCond, DenseVector<FERR> &fErr, DenseVector<BERR> &bErr,
         DenseVector<VWORK> &work, DenseVector<VIWORK> &)
{
    typedef typename GeMatrix<FS<double, cxxblas::ColMajor, I, Alloc> >::IndexType IndexType;
    const int n = int(A.numRows()), nrhs = int(B.numCols());
    const int lda = int(A.leadingDimension() > 0 ? A.leadingDimension() : 1);
    const int ldaf = int(AF.leadingDimension() > 0 ? AF.leadingDimension() : 1);
    const int ldb = int(B.leadingDimension() > 0 ? B.leadingDimension() : 1);
    const int ldx = int(X.leadingDimension() > 0 ? X.leadingDimension() : 1);
    const char f = static_cast<char>(fact), t = flens_gb300::detail::trans_char(trans);
    char eq = static_cast<char>(equed);
    std::vector<int> p = flens_gb300::detail::to_vec<int>(piv), iw(n > 0 ? n : 1);
    std::vector<double> rv = flens_gb300::detail::to_vec<double>(r);
    std::vector<double> cv = flens_gb300::detail::to_vec<double>(c);
    std::vector<double> fe(nrhs > 0 ? nrhs : 1), be(nrhs > 0 ? nrhs : 1);
    std::vector<double> w(4 * std::size_t(n > 0 ? n : 1));
    double rc = 0.0;
    int info = 0;
    dgesvx_(&f, &t, &n, &nrhs, A.data(), &lda, AF.data(), &ldaf, p.data(), &eq, rv.data(),
            cv.data(), B.data(), &ldb, X.data(), &ldx, &rc, fe.data(), be.data(), w.data(),
            iw.data(), &info);
    if (info <= -1000)
        std::fprintf(stderr, "[flens_gb300] dgesvx_ failed (%d): %s\n", info, flens_gb300_last_error());
    flens_gb300::detail::from_vec(p, piv);
    flens_gb300::detail::from_vec(rv, r);
    flens_gb300::detail::from_vec(cv, c);
    flens_gb300::detail::from_vec(fe, fErr);
    flens_gb300::detail::from_vec(be, bErr);
    rCond = rc;
    if (work.length() > 0) work(work.firstIndex()) = w[0];
    return IndexType(info);
}

} } }  // namespace generic, lapack, flens

#include <flens/flens.tcc>

#endif  // FLENS_GB300_FLENS_GB300_HPP
