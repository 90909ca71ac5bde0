// C entry points over the reference library itself (Mat-8.3.1, header-only),
// compiled unmodified from the reference tree into oracle/_ref/libmatref.so.
// Used only to validate the oracle restatement and to generate the golden
// fixtures under tests/golden/; never linked into the product.
//
// All arrays are column-major with ld = rows (Mat's MAT<T> layout).
#include "mat_prelude.h"
#include "Mat.h"

namespace {

MAT<double> make(int r, int c, const double* p) {
    MAT<double> M(r, c);
    std::memcpy(M.data, p, sizeof(double) * (size_t)r * c);
    return M;
}

void out(const MAT<double>& M, double* p) {
    std::memcpy(p, M.data, sizeof(double) * (size_t)M.rows * M.cols);
}

}  // namespace

extern "C" {

// operator* (Mat-8.3.1/Mul/Mul.h:204-235)
void ref_dgemm(int m, int n, int k, const double* A, const double* B, double* C) {
    MAT<double> a = make(m, k, A), b = make(k, n, B);
    MAT<double> c = a * b;
    out(c, C);
}

// PLU(A, pos, L, U) (Mat-8.3.1/LU/__PLU.h:152-190), outputs allocated as LU_init (Mat.h:128-131)
void ref_plu(int m, int n, const double* A, int* pos, double* L, double* U) {
    MAT<double> a = make(m, n, A), l, u;
    LU_init(a, l, u);
    // Mat never writes L's columns >= min(m, n) (they stay as allocated)
    l.fill(0.0);
    u.fill(0.0);
    PLU(a, pos, l, u);
    out(l, L);
    out(u, U);
}

// LU without pivoting (Mat-8.3.1/LU/__LU.h:71-108)
void ref_lu(int n, const double* A, double* L, double* U) {
    MAT<double> a = make(n, n, A), l, u;
    LU_init(a, l, u);
    LU(a, l, u);
    out(l, L);
    out(u, U);
}

// Solve_direct(A, B) (Mat-8.3.1/LU/__Solve_direct.h:146-220)
void ref_solve(int n, int nrhs, const double* A, const double* B, double* X) {
    MAT<double> a = make(n, n, A), b = make(n, nrhs, B);
    MAT<double> x = Solve_direct(a, b);
    out(x, X);
}

// LLT(A, L) (Mat-8.3.1/LU/__LLT.h:212-246)
void ref_llt(int n, const double* A, double* L) {
    MAT<double> a = make(n, n, A), l(n, n);
    LLT(a, l);
    out(l, L);
}

// LDLT(A, L, D) (Mat-8.3.1/LU/__LLT.h:249-295)
void ref_ldlt(int n, const double* A, double* L, double* D) {
    MAT<double> a = make(n, n, A), l(n, n), d(n, n);
    LDLT(a, l, d);
    out(l, L);
    out(d, D);
}

// QR(A, Q, R, QR_Householder) (Mat-8.3.1/QR/QR.h:8-25); Q is m x m, R is m x n
void ref_qr(int m, int n, const double* A, double* Q, double* R) {
    MAT<double> a = make(m, n, A), q, r;
    QR_init(a, q, r);
    QR(a, q, r, QR_Householder);
    out(q, Q);
    out(r, R);
}

// Det(A) (Mat-8.3.1/LU/__Det.h:30-101)
double ref_det(int n, const double* A) {
    MAT<double> a = make(n, n, A);
    return Det(a);
}

// Inv(A) (Mat-8.3.1/LU/__Inv.h:212)
void ref_inv(int n, const double* A, double* X) {
    MAT<double> a = make(n, n, A);
    MAT<double> x = Inv(a);
    out(x, X);
}

}  // extern "C"
