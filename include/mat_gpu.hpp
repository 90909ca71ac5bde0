// mat_gpu.hpp - drop-in for Mat's C++ header API (Mat-8.3.1/Mat.h) on the
// GB300 path.  Include this instead of Mat.h: it provides Mat's MAT<T> type
// with the same layout and ownership semantics (Mat-8.3.1/Base/__Matrix.h:
// column-major, ld = rows, owned `new T[]` data, swap-on-assign) and, for
// double, the hot-path calls of Mat routed through libmatgpu's C ABI:
//
//   operator*(MAT, MAT)                 Mat-8.3.1/Mul/Mul.h:204-235
//   PLU(A, pos, L, U), PLU_getP, LU_init Mat-8.3.1/LU/__PLU.h:152-197, Mat.h:128-131
//   LU(A, L, U) (no pivoting)           Mat-8.3.1/LU/__LU.h:71-108
//   LLT(A, L)                           Mat-8.3.1/LU/__LLT.h:212-246
//   LDLT(A, L, D)                       Mat-8.3.1/LU/__LLT.h:249-295
//   Solve_direct(A, B)                  Mat-8.3.1/LU/__Solve_direct.h:146-220
//   Det(A)                              Mat-8.3.1/LU/__Det.h:30-101
//   Inv(A)                              Mat-8.3.1/LU/__Inv.h:212-225
//   QR(A, Q, R, QR_Householder), QR_init Mat-8.3.1/QR/QR.h:8-25, Mat.h:132-136
//   EVD_Q(A, E, Q, eps, EVD_QR), EVD_init declared by Mat-8.3.1/Mat.h:32, 120
//                                       (defined in Mat-8.1/EVD/EVD_Q.h:7-35)
//
// plus one call Mat does not have: Solve_mixed(A, B) (mixed-precision LU with
// FP64 refinement; FP64 backward error, much faster on GB300).
//
// The matrices stay in host memory as in Mat; each call copies its operands
// to the GPU and the results back.  Errors that Mat cannot report (CUDA
// failures) throw std::runtime_error; singular / non-SPD inputs behave like
// Mat (no exception) and the library's status is kept in matgpu::last_status().
#pragma once

#include <cstddef>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>

#include "mat_gpu.h"

#ifndef XiangZiMatImport
enum QR_type { QR_Householder, QR_Givens, QR_GramSchmidt };
enum EVD_type { EVD_QR, EVD_Jacobi };
#endif

template <typename T>
class MAT {
public:
    int rows;
    int cols;
    T* data;

    MAT() : rows(0), cols(0), data(nullptr) {}
    MAT(int r, int c) : rows(r), cols(c), data(new T[(size_t)r * c]) {}
    template <class t>
    MAT(int r, int c, t* p) : rows(r), cols(c), data(new T[(size_t)r * c]) {
        for (size_t i = 0; i < (size_t)r * c; ++i) data[i] = (T)p[i];
    }
    MAT(const MAT& a) : rows(a.rows), cols(a.cols), data(new T[(size_t)a.rows * a.cols]) {
        std::memcpy(data, a.data, sizeof(T) * (size_t)rows * cols);
    }
    MAT(MAT&& a) noexcept : rows(a.rows), cols(a.cols), data(a.data) { a.data = nullptr; }
    ~MAT() { delete[] data; }

    void init(int r, int c) {
        if (rows != r || cols != c) {
            delete[] data;
            rows = r;
            cols = c;
            data = new T[(size_t)r * c];
        }
    }
    void fill(T a) {
        for (size_t i = 0; i < (size_t)rows * cols; ++i) data[i] = a;
    }
    T* operator[](int c) const { return data + (size_t)rows * c; }
    T& operator()(int r, int c) const { return data[(size_t)rows * c + r]; }
    // Mat assigns by swapping with a by-value copy (Base/__Matrix.h:149-155)
    void operator=(MAT B) {
        rows = B.rows;
        cols = B.cols;
        std::swap(data, B.data);
    }
    void operator&(MAT& B) {
        std::swap(rows, B.rows);
        std::swap(cols, B.cols);
        std::swap(data, B.data);
    }
};

namespace matgpu {

inline mg_status_t& last_status() {
    thread_local mg_status_t s = MG_OK;
    return s;
}

struct Handle {
    mg_handle_t h = nullptr;
    ~Handle() {
        if (h) mg_handle_destroy(h);
    }
};

inline mg_handle_t handle() {
    thread_local Handle hh;
    if (!hh.h) {
        mg_status_t s = mg_handle_create(&hh.h, nullptr);
        if (s != MG_OK) throw std::runtime_error(std::string("matgpu: no CUDA device: ") + mg_status_string(s));
    }
    return hh.h;
}

inline void check(mg_status_t s, const char* what) {
    last_status() = s;
    if (s == MG_OK || s == MG_SINGULAR || s == MG_NOT_SPD || s == MG_FALLBACK_USED) return;
    throw std::runtime_error(std::string("matgpu: ") + what + ": " + mg_status_string(s) + " " +
                             mg_get_last_error(handle()));
}

// Device buffer owned for the duration of one call.
struct Dev {
    void* p = nullptr;
    explicit Dev(size_t bytes) {
        if (bytes && mg_device_malloc(&p, bytes) != MG_OK) throw std::runtime_error("matgpu: device allocation");
    }
    ~Dev() {
        if (p) mg_device_free(p);
    }
    Dev(const Dev&) = delete;
    Dev& operator=(const Dev&) = delete;
    double* d() const { return (double*)p; }
};

inline void h2d(void* dst, const void* src, size_t bytes) {
    check(mg_memcpy(handle(), dst, src, bytes, 0), "copy to device");
}
inline void d2h(void* dst, const void* src, size_t bytes) {
    check(mg_memcpy(handle(), dst, src, bytes, 1), "copy to host");
    check(mg_synchronize(handle()), "synchronize");
}

}  // namespace matgpu

// C = A * B (Mat's operator* for double).
inline MAT<double> operator*(const MAT<double>& A, const MAT<double>& B) {
    MAT<double> C(A.rows, B.cols);
    const size_t sa = (size_t)A.rows * A.cols, sb = (size_t)B.rows * B.cols, sc = (size_t)C.rows * C.cols;
    if (sc == 0) return C;
    matgpu::Dev dA(sa * 8), dB(sb * 8), dC(sc * 8);
    matgpu::h2d(dA.p, A.data, sa * 8);
    matgpu::h2d(dB.p, B.data, sb * 8);
    matgpu::check(mg_dgemm(matgpu::handle(), 0, 0, A.rows, B.cols, A.cols, 1.0, dA.d(), A.rows > 1 ? A.rows : 1,
                           dB.d(), B.rows > 1 ? B.rows : 1, 0.0, dC.d(), C.rows > 1 ? C.rows : 1),
                  "mg_dgemm");
    matgpu::d2h(C.data, dC.p, sc * 8);
    return C;
}

// C = A * B for MAT<float> (the same operator* template in Mat).  Products
// with k >= 32 and m n k >= 2^27 run on the tensor cores as split-BF16 (3
// terms, lower-order products first, fp32 accumulation: fp32-class accuracy),
// the rest on the FP32 SIMT GEMM.
inline MAT<float> operator*(const MAT<float>& A, const MAT<float>& B) {
    MAT<float> C(A.rows, B.cols);
    const size_t sa = (size_t)A.rows * A.cols, sb = (size_t)B.rows * B.cols, sc = (size_t)C.rows * C.cols;
    if (sc == 0) return C;
    matgpu::Dev dA(sa * 4), dB(sb * 4), dC(sc * 4);
    matgpu::h2d(dA.p, A.data, sa * 4);
    matgpu::h2d(dB.p, B.data, sb * 4);
    const int lda = A.rows > 1 ? A.rows : 1, ldb = B.rows > 1 ? B.rows : 1, ldc = C.rows > 1 ? C.rows : 1;
    if (A.cols >= 32 && (double)A.rows * B.cols * A.cols >= (double)(1 << 27))
        matgpu::check(mg_sgemm_bf16x_ex(matgpu::handle(), 3, MG_BF16X_ORDERED, A.rows, B.cols, A.cols, 1.0f,
                                        (const float*)dA.p, lda, (const float*)dB.p, ldb, 0.0f, (float*)dC.p, ldc),
                      "mg_sgemm_bf16x_ex");
    else
        matgpu::check(mg_sgemm(matgpu::handle(), 0, 0, A.rows, B.cols, A.cols, 1.0f, (const float*)dA.p, lda,
                               (const float*)dB.p, ldb, 0.0f, (float*)dC.p, ldc),
                      "mg_sgemm");
    matgpu::d2h(C.data, dC.p, sc * 4);
    return C;
}

template <typename t1, typename t2>
void LU_init(MAT<t1>& A, MAT<t2>& L, MAT<t2>& U) {
    L.init(A.rows, A.rows);
    U.init(A.rows, A.cols);
}

template <typename t1, typename t2>
void QR_init(MAT<t1>& A, MAT<t2>& Q, MAT<t2>& R) {
    Q.init(A.rows, A.rows);
    R.init(A.rows, A.cols);
}

// PLU(A, pos, L, U): A(pos[i], :) = (L U)(i, :), L unit lower (m x m), U upper (m x n).
inline void PLU(MAT<double>& A, int* pos, MAT<double>& L, MAT<double>& U) {
    const int m = A.rows, n = A.cols, s = m < n ? m : n;
    const size_t sa = (size_t)m * n;
    if (sa == 0) return;
    matgpu::Dev dA(sa * 8), dpos((size_t)m * sizeof(int));
    matgpu::h2d(dA.p, A.data, sa * 8);
    int info = 0;
    matgpu::check(mg_dgetrf(matgpu::handle(), m, n, dA.d(), m, (int*)dpos.p, &info), "mg_dgetrf");
    MAT<double> LU(m, n);
    matgpu::d2h(LU.data, dA.p, sa * 8);
    matgpu::d2h(pos, dpos.p, (size_t)m * sizeof(int));
    L.init(m, m);
    U.init(m, n);
    std::memset(L.data, 0, sizeof(double) * (size_t)m * m);
    std::memcpy(U.data, LU.data, sizeof(double) * sa);
    for (int c = 0; c < s; ++c) {
        L(c, c) = 1.0;
        for (int r = c + 1; r < m; ++r) {
            L(r, c) = LU(r, c);
            U(r, c) = 0.0;
        }
    }
}

template <typename t>
void PLU_getP(int* pos, MAT<t>& P) {
    std::memset(P.data, 0, sizeof(t) * (size_t)P.rows * P.cols);
    for (int i = 0; i < P.rows; ++i) P(pos[i], i) = 1;
}

// LU(A, L, U) without pivoting (square A, L and U allocated as LU_init does):
// L unit lower, U upper, bit for bit Mat's.
inline void LU(MAT<double>& A, MAT<double>& L, MAT<double>& U) {
    const int n = A.rows;
    L.init(n, n);
    U.init(n, n);
    if (n == 0) return;
    matgpu::Dev dA((size_t)n * n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    int info = 0;
    matgpu::check(mg_dlu(matgpu::handle(), n, dA.d(), n, &info), "mg_dlu");
    MAT<double> F(n, n);
    matgpu::d2h(F.data, dA.p, (size_t)n * n * 8);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
            L(r, c) = r > c ? F(r, c) : (r == c ? 1.0 : 0.0);
            U(r, c) = r <= c ? F(r, c) : 0.0;
        }
}

// LLT(A, L): reads the lower triangle of A; L lower, strict upper zeroed.
inline void LLT(MAT<double>& A, MAT<double>& L) {
    const int n = A.rows;
    L.init(n, n);
    if (n == 0) return;
    matgpu::Dev dA((size_t)n * n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    int info = 0;
    matgpu::check(mg_dpotrf(matgpu::handle(), n, dA.d(), n, &info), "mg_dpotrf");
    matgpu::d2h(L.data, dA.p, (size_t)n * n * 8);
}

// LDLT(A, L, D): reads the lower triangle of A; L lower (diagonal as Mat
// leaves it, d_j * (1/d_j)), strict upper zeroed; D = diag(d).
inline void LDLT(MAT<double>& A, MAT<double>& L, MAT<double>& D) {
    const int n = A.rows;
    L.init(n, n);
    D.init(n, n);
    if (n == 0) return;
    matgpu::Dev dA((size_t)n * n * 8), dd((size_t)n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    int info = 0;
    matgpu::check(mg_dldlt(matgpu::handle(), n, dA.d(), n, (double*)dd.p, &info), "mg_dldlt");
    matgpu::d2h(L.data, dA.p, (size_t)n * n * 8);
    MAT<double> d(n, 1);
    matgpu::d2h(d.data, dd.p, (size_t)n * 8);
    std::memset(D.data, 0, sizeof(double) * (size_t)n * n);
    for (int i = 0; i < n; ++i) D(i, i) = d.data[i];
}

// LLT on MAT<float>.
inline void LLT(MAT<float>& A, MAT<float>& L) {
    const int n = A.rows;
    L.init(n, n);
    if (n == 0) return;
    matgpu::Dev dA((size_t)n * n * 4);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 4);
    int info = 0;
    matgpu::check(mg_spotrf(matgpu::handle(), n, (float*)dA.p, n, &info), "mg_spotrf");
    matgpu::d2h(L.data, dA.p, (size_t)n * n * 4);
}

// QR(A, Q, R, QR_Householder): Q (m x m) and R (m x n) as Mat forms them
// (blocked Householder).  Givens and Gram-Schmidt are not on the GPU.
inline void QR(MAT<double>& A, MAT<double>& Q, MAT<double>& R, QR_type type) {
    if (type != QR_Householder) throw std::runtime_error("mat_gpu: QR supports QR_Householder only");
    const int m = A.rows, n = A.cols;
    Q.init(m, m);
    R.init(m, n);
    if ((size_t)m * n == 0) return;
    matgpu::Dev dA((size_t)m * n * 8), dQ((size_t)m * m * 8), dR((size_t)m * n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)m * n * 8);
    matgpu::check(mg_dqr(matgpu::handle(), m, n, dA.d(), m, dQ.d(), m, dR.d(), m), "mg_dqr");
    matgpu::d2h(Q.data, dQ.p, (size_t)m * m * 8);
    matgpu::d2h(R.data, dR.p, (size_t)m * n * 8);
}

template <typename t1, typename t2>
void EVD_init(MAT<t1>& A, MAT<t2>& E, MAT<t2>& X) {
    E.init(A.rows, A.rows);
    X.init(A.rows, A.rows);
}

// EVD_Q(A, E, Q, eps, EVD_QR) of symmetric A (its lower triangle is read):
// E = diag(eigenvalues), Q the eigenvectors (A Q = Q E), bit for bit the
// Mat-8.1 snapshot's result (Householder tridiagonalisation, implicit QR
// sweeps with absolute deflation threshold eps).  Mat iterates without limit;
// here a matrix that does not deflate within 64 n sweeps throws.
inline void EVD_Q(MAT<double>& A, MAT<double>& E, MAT<double>& Q, double eps, EVD_type type) {
    if (type != EVD_QR) throw std::runtime_error("mat_gpu: EVD_Q supports EVD_QR only");
    const int n = A.rows;
    EVD_init(A, E, Q);
    if (n == 0) return;
    matgpu::Dev dA((size_t)n * n * 8), dE((size_t)n * n * 8), dQ((size_t)n * n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    matgpu::check(mg_devd_q(matgpu::handle(), n, dA.d(), n, eps, dE.d(), n, dQ.d(), n, nullptr), "mg_devd_q");
    matgpu::d2h(E.data, dE.p, (size_t)n * n * 8);
    matgpu::d2h(Q.data, dQ.p, (size_t)n * n * 8);
}

// X = A^{-1} B (A taken by value, as in Mat).
inline MAT<double> Solve_direct(MAT<double> A, MAT<double>& B) {
    const int n = A.rows, k = B.cols;
    MAT<double> X(n, k);
    if ((size_t)n * k == 0) return X;
    matgpu::Dev dA((size_t)n * n * 8), dB((size_t)n * k * 8), dX((size_t)n * k * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    matgpu::h2d(dB.p, B.data, (size_t)n * k * 8);
    int info = 0;
    matgpu::check(mg_dgesv(matgpu::handle(), n, k, dA.d(), n, dB.d(), n, dX.d(), n, &info), "mg_dgesv");
    matgpu::d2h(X.data, dX.p, (size_t)n * k * 8);
    return X;
}

// Mixed-precision solve (no counterpart in Mat): same result quality as
// Solve_direct (FP64 normwise backward error <= 1e-14), much faster on GB300.
inline MAT<double> Solve_mixed(MAT<double>& A, MAT<double>& B, mg_ir_report* report = nullptr) {
    const int n = A.rows, k = B.cols;
    MAT<double> X(n, k);
    if ((size_t)n * k == 0) return X;
    matgpu::Dev dA((size_t)n * n * 8), dB((size_t)n * k * 8), dX((size_t)n * k * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    matgpu::h2d(dB.p, B.data, (size_t)n * k * 8);
    mg_ir_report rep;
    matgpu::check(mg_dsgesv_ir(matgpu::handle(), n, k, dA.d(), n, dB.d(), n, dX.d(), n, nullptr, &rep),
                  "mg_dsgesv_ir");
    if (report) *report = rep;
    matgpu::d2h(X.data, dX.p, (size_t)n * k * 8);
    return X;
}

// Det(A) (Mat's Det: PLU, permutation parity, product of U's diagonal in order).
inline double Det(MAT<double> A) {
    const int n = A.rows;
    if (n == 0) return 1.0;
    matgpu::Dev dA((size_t)n * n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    double d = 0.0;
    matgpu::check(mg_ddet(matgpu::handle(), n, dA.d(), n, &d), "mg_ddet");
    return d;
}

// Inv(A) (A taken by value, as in Mat), bit for bit Mat's result.
inline MAT<double> Inv(MAT<double> A) {
    const int n = A.rows;
    MAT<double> X(n, n);
    if (n == 0) return X;
    matgpu::Dev dA((size_t)n * n * 8), dX((size_t)n * n * 8);
    matgpu::h2d(dA.p, A.data, (size_t)n * n * 8);
    int info = 0;
    matgpu::check(mg_dinv(matgpu::handle(), n, dA.d(), n, dX.d(), n, &info), "mg_dinv");
    matgpu::d2h(X.data, dX.p, (size_t)n * n * 8);
    return X;
}
