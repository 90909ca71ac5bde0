// Mat call sites compiled against the drop-in header (include/mat_gpu.hpp)
// instead of Mat.h; writes every result to <outdir>/<name>.bin (raw doubles /
// ints) for the Python test to compare with the oracle.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "mat_gpu.hpp"

static std::string dir;

template <typename T>
static void dump(const char* name, const T* p, size_t n) {
    FILE* f = std::fopen((dir + "/" + name + ".bin").c_str(), "wb");
    if (!f) std::exit(3);
    std::fwrite(p, sizeof(T), n, f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    dir = argv[1];
    // the same seeded inputs the test regenerates in Python
    MAT<double> A(150, 130), B(130, 170);
    mg_host_fill_uniform(A.data, A.rows, A.cols, A.rows, 0, -1.0, 1.0, 1);
    mg_host_fill_uniform(B.data, B.rows, B.cols, B.rows, 1, -1.0, 1.0, 1);
    MAT<double> C = A * B;
    dump("gemm", C.data, (size_t)C.rows * C.cols);

    MAT<double> G(300, 300), L, U;
    mg_host_fill_normal(G.data, 300, 300, 300, 2, 1);
    int pos[300];
    LU_init(G, L, U);
    PLU(G, pos, L, U);
    dump("plu_pos", pos, 300);
    dump("plu_L", L.data, (size_t)L.rows * L.cols);
    dump("plu_U", U.data, (size_t)U.rows * U.cols);

    // LU without pivoting on a diagonally dominant matrix
    MAT<double> Gd(200, 200), Ln, Un;
    mg_host_fill_normal(Gd.data, 200, 200, 200, 4, 1);
    for (int i = 0; i < 200; ++i) Gd(i, i) += 200.0;
    LU(Gd, Ln, Un);
    dump("lu_L", Ln.data, (size_t)200 * 200);
    dump("lu_U", Un.data, (size_t)200 * 200);

    MAT<double> b(300, 3);
    mg_host_fill_normal(b.data, 300, 3, 300, 3, 1);
    MAT<double> x = Solve_direct(G, b);
    dump("solve", x.data, (size_t)x.rows * x.cols);
    MAT<double> bw(300, 10);  // wide path (more than 4 right-hand sides)
    mg_host_fill_normal(bw.data, 300, 10, 300, 8, 1);
    MAT<double> xw = Solve_direct(G, bw);
    dump("solve_wide", xw.data, (size_t)xw.rows * xw.cols);
    MAT<double> xm = Solve_mixed(G, b);
    dump("solve_mixed", xm.data, (size_t)xm.rows * xm.cols);

    double d = Det(G);
    dump("det", &d, 1);
    MAT<double> Gi = Inv(G);
    dump("inv", Gi.data, (size_t)300 * 300);

    // S = W W^T / n + I from the same generator, computed with the drop-in product
    MAT<double> W(200, 200), Wt(200, 200), S;
    mg_host_fill_normal(W.data, 200, 200, 200, 4, 1);
    for (int i = 0; i < 200; ++i)
        for (int j = 0; j < 200; ++j) Wt(i, j) = W(j, i);
    S = W * Wt;
    for (int i = 0; i < 200 * 200; ++i) S.data[i] /= 200.0;
    for (int i = 0; i < 200; ++i) S(i, i) += 1.0;
    dump("spd", S.data, (size_t)200 * 200);
    MAT<double> Lc(200, 200);
    LLT(S, Lc);
    dump("llt", Lc.data, (size_t)200 * 200);
    MAT<double> Ld, Dd;
    LDLT(S, Ld, Dd);
    dump("ldlt_L", Ld.data, (size_t)200 * 200);
    dump("ldlt_D", Dd.data, (size_t)200 * 200);
    // QR(A, Q, R, QR_Householder), blocked path (min(m, n) > 96)
    MAT<double> Aq(300, 200), Q, R;
    mg_host_fill_normal(Aq.data, 300, 200, 300, 7, 1);
    QR_init(Aq, Q, R);
    QR(Aq, Q, R, QR_Householder);
    dump("qr_Q", Q.data, (size_t)300 * 300);
    dump("qr_R", R.data, (size_t)300 * 200);

    // EVD_Q(A, E, Q, eps, EVD_QR) of the symmetric W + W^T
    MAT<double> Sy(150, 150), Ev, Qv;
    for (int i = 0; i < 150; ++i)
        for (int j = 0; j < 150; ++j) Sy(i, j) = W(i, j) + W(j, i);
    EVD_init(Sy, Ev, Qv);
    EVD_Q(Sy, Ev, Qv, 1e-10, EVD_QR);
    dump("evd_E", Ev.data, (size_t)150 * 150);
    dump("evd_Q", Qv.data, (size_t)150 * 150);

    // operator* on MAT<float>
    MAT<float> Fa(70, 50), Fb(50, 60);
    for (int i = 0; i < 70 * 50; ++i) Fa.data[i] = (float)A.data[i];
    for (int i = 0; i < 50 * 60; ++i) Fb.data[i] = (float)B.data[i];
    MAT<float> Fc = Fa * Fb;
    dump("sgemm", Fc.data, (size_t)70 * 60);
    std::printf("ok\n");
    return 0;
}
