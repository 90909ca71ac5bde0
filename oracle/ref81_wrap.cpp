// C entry points over the Mat-8.1 snapshot's symmetric tridiagonalisation
// (EVD/__QR.h) and the QR iteration that follows it, compiled unmodified from
// the reference tree into oracle/_ref/libmat81ref.so.  Used only to validate
// the oracle restatement and to generate the golden fixtures under
// tests/golden/; never linked into the product.
//
// Arrays are column-major with ld = rows (Mat's MAT<T> layout).
#include "mat81_prelude.h"
#include "SIMD/SIMD.h"
#include "Base/Base.h"
#include "QR/__Householder.h"
#include "QR/__Givens.h"
#include "EVD/__QR.h"

extern "C" {

// __EVD_Q_Householder(Q, R, v) (Mat-8.1/EVD/__QR.h:2-47): R holds the
// symmetric matrix on entry; on return d = R's last column (diagonal of the
// tridiagonal matrix, n entries), e = the n-1 entries from R(1, n-2) (its
// off-diagonal), Q the orthogonal factor formed by __Householder_Q2.
void ref81_tridiag(int n, const double* A, double* Q, double* d, double* e) {
    MAT<double> R(n, n), q(n, n);
    std::memcpy(R.data, A, sizeof(double) * (size_t)n * n);
    std::memset(q.data, 0, sizeof(double) * (size_t)n * n);
    double* v = new double[n + 8];
    __EVD_Q_Householder(q, R, v);
    delete[] v;
    std::memcpy(Q, q.data, sizeof(double) * (size_t)n * n);
    std::memcpy(d, R[n - 1], sizeof(double) * (size_t)n);
    std::memcpy(e, R[n - 2] + 1, sizeof(double) * (size_t)(n - 1));
}

// EVD_Q(A, E, Q, eps, EVD_QR) (Mat-8.1/EVD/EVD_Q.h:7-35 -> EVD/__QR.h:145-169)
void ref81_evd_q(int n, const double* A, double eps, double* E, double* Q) {
    MAT<double> a(n, n), e(n, n), q(n, n);
    std::memcpy(a.data, A, sizeof(double) * (size_t)n * n);
    std::memset(q.data, 0, sizeof(double) * (size_t)n * n);
    __copy(e.data, a.data, n * n);
    __EVD_Q_QR(e, q, eps);
    std::memcpy(E, e.data, sizeof(double) * (size_t)n * n);
    std::memcpy(Q, q.data, sizeof(double) * (size_t)n * n);
}

}  // extern "C"
