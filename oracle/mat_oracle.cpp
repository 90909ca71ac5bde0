// ORACLE — test infrastructure only.  A CPU restatement of Mat-8.3.1's
// algorithms for the GPU hot path (GEMM, blocked PLU, Solve_direct, blocked
// LLT, blocked Householder QR, Det, Inv), written from the reference's behaviour,
// with each routine citing the reference file:line it follows.  Only the
// tests, the smoke check and the benchmark's CPU-baseline leg may load it.
//
// Numerics follow Mat's AVX-512 double build: every multiply-add is a fused
// fma in the same per-element order (sequential over k for the GEMM
// updates, Mat-8.3.1/Mul/__micro_kernel_packed_double.h:43-84; fmadd for
// __mixed, Calculate/__AVX512_double.h:81-93), reciprocals where Mat
// multiplies by 1/x, and the same first-index-of-max pivot rule
// (LU/__PLU.h:67-77).  Parity with the reference itself is checked by the
// CPU tests against oracle/_ref (the reference compiled from its headers)
// and against the committed golden fixtures.
//
// All matrices are column-major with an explicit leading dimension.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

// The seeded input streams (counter-based, bit-identical on the host and the
// GPU) are the library's; the oracle generates the same inputs from them.
#include "../mat_gb300/csrc/rng.cuh"

namespace {

int g_threads = 1;

// Block sizes of Mat's AVX-512 configuration (Mat-8.3.1/Mat.h:57-81).
constexpr int BS_LU = 60;
constexpr int BS_LLT = 48;
constexpr int BS_QR = 48;

inline double& at(double* A, int lda, int r, int c) { return A[r + (size_t)c * lda]; }

// ------------------------------------------------------------ host threads
// The reference is single-threaded; the restatement spreads independent
// elements over host threads without changing any element's operation
// sequence, so its results do not depend on the thread count.
//
// Pool: persistent workers; run(nt, fn) calls fn(tid, nt) on nt threads (the
// caller is thread 0) and returns when all have finished.  A pool created
// before a fork() is rebuilt in the child (its workers did not survive).
class Pool {
public:
    ~Pool() { stop(); }

    void run(int nt, const std::function<void(int, int)>& fn) {
        nt = std::max(1, nt);
        if (nt == 1 || in_job()) {  // nested inside a job: run inline
            fn(0, 1);
            return;
        }
        std::lock_guard<std::mutex> serial(run_mu_);
        {
            std::lock_guard<std::mutex> g(mu_);
            ensure(nt - 1);
            job_ = &fn;
            job_nt_ = nt;
            pending_ = nt - 1;
            ++gen_;
        }
        cv_.notify_all();
        in_job() = true;
        fn(0, nt);
        in_job() = false;
        std::unique_lock<std::mutex> g(mu_);
        done_cv_.wait(g, [&] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    static bool& in_job() {
        static thread_local bool flag = false;
        return flag;
    }
    // called with mu_ held, before the job's generation is published: a new
    // worker starts from the current generation and so sees the next job
    void ensure(int workers) {
        if (pid_ != getpid()) {  // after a fork: the old workers do not exist here
            for (auto& t : th_) t.detach();
            th_.clear();
            pid_ = getpid();
            quit_ = false;
        }
        while ((int)th_.size() < workers) {
            const int id = (int)th_.size() + 1;
            const uint64_t start = gen_;
            th_.emplace_back([this, id, start] { loop(id, start); });
        }
    }
    void loop(int id, uint64_t seen) {
        in_job() = true;
        for (;;) {
            const std::function<void(int, int)>* job = nullptr;
            int nt = 0;
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return quit_ || gen_ != seen; });
                if (quit_) return;
                seen = gen_;
                job = job_;
                nt = job_nt_;
            }
            if (id < nt) {
                (*job)(id, nt);
                std::lock_guard<std::mutex> g(mu_);
                if (--pending_ == 0) done_cv_.notify_all();
            }
        }
    }
    void stop() {
        {
            std::lock_guard<std::mutex> g(mu_);
            quit_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_)
            if (t.joinable()) {
                if (pid_ == getpid())
                    t.join();
                else
                    t.detach();
            }
    }

    std::vector<std::thread> th_;
    std::mutex mu_, run_mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int, int)>* job_ = nullptr;
    int job_nt_ = 0, pending_ = 0;
    uint64_t gen_ = 0;
    bool quit_ = false;
    pid_t pid_ = getpid();
};

Pool& pool() {
    static Pool p;
    return p;
}

// Sense-reversing spin barrier for phases inside one Pool::run.
class SpinBarrier {
public:
    explicit SpinBarrier(int n) : n_(n) {}
    void wait() {
        const int ph = phase_.load(std::memory_order_acquire);
        if (count_.fetch_add(1, std::memory_order_acq_rel) == n_ - 1) {
            count_.store(0, std::memory_order_relaxed);
            phase_.store(ph + 1, std::memory_order_release);
            return;
        }
        for (unsigned spins = 0; phase_.load(std::memory_order_acquire) == ph; ++spins)
            if ((spins & 1023u) == 1023u) std::this_thread::yield();
    }

private:
    const int n_;
    std::atomic<int> count_{0};
    std::atomic<int> phase_{0};
};

// Splits [0, n) into nt contiguous chunks; chunk t is [lo, hi).
inline void chunk(int n, int t, int nt, int& lo, int& hi) {
    const int q = n / nt, r = n % nt;
    lo = t * q + std::min(t, r);
    hi = lo + q + (t < r ? 1 : 0);
}

// Runs fn(lo, hi) over [0, n) split into contiguous chunks across threads.
void parallel_cols(int n, const std::function<void(int, int)>& fn) {
    const int t = std::max(1, std::min(g_threads, n));
    pool().run(t, [&](int tid, int nt) {
        int lo, hi;
        chunk(n, tid, nt, lo, hi);
        if (lo < hi) fn(lo, hi);
    });
}

// ------------------------------------------------------------------ GEMM
// C(m x n) (+|-)= A(m x k) * op(B): per element a sequential fused chain over
// p = 0..k-1 starting from C (Mat's micro-kernels load C and fmadd / fnmadd
// into it, Mul/__micro_kernel_packed_double.h:14-110 and :301-398; fnmadd
// c - a b is fma(a, -b, c)).  Mat's own KC blocking stores the partial chain
// to C and reloads it, which changes nothing, and neither does the blocking
// here: A is packed in slivers of MR rows, op(B) (negated when subtracting)
// in slivers of NR columns, per KC block of k; an MR x NR register tile runs
// each element's chain over the block; tiles are spread over the threads.
constexpr int MR = 8, NR = 6, KC = 256;
constexpr int TILE_MS = 16, TILE_NS = 16;  // slivers per tile: 128 rows x 96 columns

// Full MR x NR tile read from and written to C in place.
inline void ukernel_c(int kc, const double* __restrict ap, const double* __restrict bp, double* __restrict c,
                      int ldc) {
    double acc[NR][MR];
    for (int j = 0; j < NR; ++j)
        for (int i = 0; i < MR; ++i) acc[j][i] = c[i + (size_t)j * ldc];
    for (int p = 0; p < kc; ++p) {
        const double* a = ap + (size_t)p * MR;
        const double* b = bp + (size_t)p * NR;
#pragma GCC unroll 8
        for (int j = 0; j < NR; ++j) {
            const double bj = b[j];
#pragma GCC unroll 8
            for (int i = 0; i < MR; ++i) acc[j][i] = std::fma(a[i], bj, acc[j][i]);
        }
    }
    for (int j = 0; j < NR; ++j)
        for (int i = 0; i < MR; ++i) c[i + (size_t)j * ldc] = acc[j][i];
}

// transB: op(B) = B^T with B given as n x k rows (ld ldb).
void gemm_core(int m, int n, int k, const double* A, int lda, const double* B, int ldb, bool transB, double* C,
               int ldc, bool subtract) {
    if (m <= 0 || n <= 0 || k <= 0) return;
    auto bval = [&](int p, int j) { return transB ? B[j + (size_t)p * ldb] : B[p + (size_t)j * ldb]; };
    if ((double)m * n * k < 4.0e5 || m < MR) {
        for (int j = 0; j < n; ++j) {
            double* c = C + (size_t)j * ldc;
            for (int p = 0; p < k; ++p) {
                const double b = subtract ? -bval(p, j) : bval(p, j);
                const double* a = A + (size_t)p * lda;
                for (int i = 0; i < m; ++i) c[i] = std::fma(a[i], b, c[i]);
            }
        }
        return;
    }
    const int ms = (m + MR - 1) / MR, ns = (n + NR - 1) / NR;
    const int nrb = (ms + TILE_MS - 1) / TILE_MS, ncb = (ns + TILE_NS - 1) / TILE_NS;
    const int kcmax = std::min(KC, k);
    std::vector<double> Ap((size_t)ms * kcmax * MR), Bp((size_t)ns * kcmax * NR);
    const int nt = std::max(1, std::min(g_threads, nrb * ncb));
    for (int p0 = 0; p0 < k; p0 += KC) {
        const int kc = std::min(KC, k - p0);
        std::atomic<int> next{0};
        SpinBarrier bar(nt);
        pool().run(nt, [&](int tid, int nth) {
            int lo, hi;
            chunk(ms, tid, nth, lo, hi);
            for (int s = lo; s < hi; ++s) {
                double* dst = Ap.data() + (size_t)s * kc * MR;
                const int r0 = s * MR, rows = std::min(MR, m - r0);
                for (int p = 0; p < kc; ++p) {
                    const double* src = A + r0 + (size_t)(p0 + p) * lda;
                    for (int i = 0; i < rows; ++i) dst[(size_t)p * MR + i] = src[i];
                    for (int i = rows; i < MR; ++i) dst[(size_t)p * MR + i] = 0.0;
                }
            }
            chunk(ns, tid, nth, lo, hi);
            for (int t = lo; t < hi; ++t) {
                double* dst = Bp.data() + (size_t)t * kc * NR;
                const int c0 = t * NR, cols = std::min(NR, n - c0);
                for (int j = 0; j < NR; ++j)
                    for (int p = 0; p < kc; ++p) {
                        double v = j < cols ? bval(p0 + p, c0 + j) : 0.0;
                        dst[(size_t)p * NR + j] = subtract ? -v : v;
                    }
            }
            bar.wait();
            for (int tile = next.fetch_add(1); tile < nrb * ncb; tile = next.fetch_add(1)) {
                const int cb = tile / nrb, rb = tile % nrb;
                const int t1 = std::min(ns, (cb + 1) * TILE_NS), s1 = std::min(ms, (rb + 1) * TILE_MS);
                for (int t = cb * TILE_NS; t < t1; ++t) {
                    const double* bp = Bp.data() + (size_t)t * kc * NR;
                    const int c0 = t * NR, cols = std::min(NR, n - c0);
                    for (int s = rb * TILE_MS; s < s1; ++s) {
                        const double* ap = Ap.data() + (size_t)s * kc * MR;
                        const int r0 = s * MR, rows = std::min(MR, m - r0);
                        double* c = C + r0 + (size_t)c0 * ldc;
                        if (rows == MR && cols == NR) {
                            ukernel_c(kc, ap, bp, c, ldc);
                        } else {
                            double buf[MR * NR] = {0};
                            for (int j = 0; j < cols; ++j)
                                for (int i = 0; i < rows; ++i) buf[i + j * MR] = c[i + (size_t)j * ldc];
                            ukernel_c(kc, ap, bp, buf, MR);
                            for (int j = 0; j < cols; ++j)
                                for (int i = 0; i < rows; ++i) c[i + (size_t)j * ldc] = buf[i + j * MR];
                        }
                    }
                }
            }
        });
    }
}

void gemm_acc(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
              bool subtract) {
    gemm_core(m, n, k, A, lda, B, ldb, false, C, ldc, subtract);
}

// C -= A * B^T with B given as rows (Mat's __times_A_BT_LLT, LU/__LLT.h:59-91).
void gemm_abt_sub(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc) {
    gemm_core(m, n, k, A, lda, B, ldb, true, C, ldc, true);
}

// Mat's AVX-512 dot product (Calculate/__AVX512_double.h:110-133): four
// 8-lane fused accumulators over 32-element strides, then the full 8-blocks
// into the first, a lane-wise (a0+a1)+(a2+a3), a masked fused tail and a
// 8 -> 4 -> 2 -> 1 horizontal reduction.
double dot_mat(const double* a, const double* b, int len) {
    double acc[4][8] = {{0}};
    const int nb = len / 8;
    int i = 0;
    for (; i <= nb - 4; i += 4)
        for (int q = 0; q < 4; ++q)
            for (int l = 0; l < 8; ++l) acc[q][l] = std::fma(a[(i + q) * 8 + l], b[(i + q) * 8 + l], acc[q][l]);
    for (; i < nb; ++i)
        for (int l = 0; l < 8; ++l) acc[0][l] = std::fma(a[i * 8 + l], b[i * 8 + l], acc[0][l]);
    double s[8];
    for (int l = 0; l < 8; ++l) s[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
    const int rem = len - nb * 8;
    for (int l = 0; l < rem; ++l) s[l] = std::fma(a[nb * 8 + l], b[nb * 8 + l], s[l]);
    double h4[4], h2[2];
    for (int l = 0; l < 4; ++l) h4[l] = s[l] + s[l + 4];
    for (int l = 0; l < 2; ++l) h2[l] = h4[l] + h4[l + 2];
    return h2[0] + h2[1];
}

// Mat's generic __dot template (Calculate/Calculate.h:266-281) as the
// reference build evaluates it (g++ 13 -O3 with AVX-512/FMA): four partial
// sums over i mod 4; the first floor(n4/32)*32 elements are vectorised with
// separate multiply and add, the remaining groups of four are fused; then
// ((t0 + t1) + t2) + t3 and a fused tail.  Overload resolution picks this
// template wherever Mat passes const pointers, e.g. CalculateT
// (QR/__Householder_Blocked.h:95), instead of the AVX-512 overload.
double dot_generic(const double* a, const double* b, int len) {
    double t0 = 0, t1 = 0, t2 = 0, t3 = 0;
    const int n4 = 4 * (len / 4), nv = (n4 / 32) * 32;
    int i = 0;
    for (; i < nv; i += 4) {
        t0 = t0 + a[i] * b[i];
        t1 = t1 + a[i + 1] * b[i + 1];
        t2 = t2 + a[i + 2] * b[i + 2];
        t3 = t3 + a[i + 3] * b[i + 3];
    }
    for (; i < n4; i += 4) {
        t0 = std::fma(a[i], b[i], t0);
        t1 = std::fma(a[i + 1], b[i + 1], t1);
        t2 = std::fma(a[i + 2], b[i + 2], t2);
        t3 = std::fma(a[i + 3], b[i + 3], t3);
    }
    double ans = t0 + t1 + t2 + t3;
    for (int j = n4; j < len; ++j) ans = std::fma(a[j], b[j], ans);
    return ans;
}

// ---------------------------------------------------------------- TRSM
// X(k x n) := L^{-1} X, L unit lower k x k (Mat's AVX-512 __Solve_direct_LX,
// LU/__Base.h:95-208): 8-column blocks by four partial sums, the ragged
// columns by column-oriented fused updates.
void trsm_lx(int k, int n, const double* L, int ldl, double* X, int ldx) {
    const int nb8 = n / 8;
    std::vector<double> nl((size_t)k * k);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < i; ++j) nl[(size_t)i * k + j] = -L[i + (size_t)j * ldl];
    // every column is independent: the 8-column blocks and the ragged tail are spread over threads
    auto cols = [&](int b0, int b1) {
        for (int b = b0; b < b1; ++b) {
            if (b < nb8) {
                // the 8 columns packed row by row (xb[j][r]), L's rows negated
                // (nl[i][j] = -L(i,j)): the same four partial chains per element
                // (j mod 4, in order) as Mat's 8-column register solve
                const int c = 8 * b;
                double xb[8 * 64 * 2];
                std::vector<double> big;
                double* x8 = xb;
                if (k > 128) {
                    big.resize((size_t)8 * k);
                    x8 = big.data();
                }
                for (int r = 0; r < 8; ++r)
                    for (int i = 0; i < k; ++i) x8[i * 8 + r] = X[i + (size_t)(c + r) * ldx];
                for (int i = 0; i < k; ++i) {
                    const double* li = nl.data() + (size_t)i * k;
                    double s0[8], s1[8], s2[8], s3[8];
                    for (int r = 0; r < 8; ++r) {
                        s0[r] = x8[i * 8 + r];
                        s1[r] = s2[r] = s3[r] = 0.0;
                    }
                    int j = 0;
                    for (; j + 4 <= i; j += 4) {
                        const double l0 = li[j], l1 = li[j + 1], l2 = li[j + 2], l3 = li[j + 3];
                        const double* x0 = x8 + j * 8;
                        for (int r = 0; r < 8; ++r) {
                            s0[r] = std::fma(l0, x0[r], s0[r]);
                            s1[r] = std::fma(l1, x0[8 + r], s1[r]);
                            s2[r] = std::fma(l2, x0[16 + r], s2[r]);
                            s3[r] = std::fma(l3, x0[24 + r], s3[r]);
                        }
                    }
                    for (; j < i; ++j)
                        for (int r = 0; r < 8; ++r) s0[r] = std::fma(li[j], x8[j * 8 + r], s0[r]);
                    for (int r = 0; r < 8; ++r) x8[i * 8 + r] = s0[r] + (s1[r] + (s2[r] + s3[r]));
                }
                for (int r = 0; r < 8; ++r)
                    for (int i = 0; i < k; ++i) X[i + (size_t)(c + r) * ldx] = x8[i * 8 + r];
            } else {
                for (int c = 8 * nb8; c < n; ++c) {
                    double* x = X + (size_t)c * ldx;
                    for (int i = 1; i < k; ++i) {
                        const double a = x[i - 1];
                        if (a == 0.0) continue;
                        const double* li = L + (size_t)(i - 1) * ldl;
                        for (int r = i; r < k; ++r) x[r] = std::fma(li[r], -a, x[r]);
                    }
                }
            }
        }
    };
    const int nblocks = nb8 + (n % 8 ? 1 : 0);
    if ((double)nblocks * k * k < 2.0e5)
        cols(0, nblocks);
    else
        parallel_cols(nblocks, cols);
}

// X(k x n) := U^{-1} X, U upper k x k (generic __Solve_direct_UX, LU/__Base.h:51-92).
void trsm_ux(int k, int n, const double* U, int ldu, double* X, int ldx) {
    for (int c = 0; c < n; ++c) {
        double* x = X + (size_t)c * ldx;
        for (int i = k - 1; i >= 0; --i) {
            x[i] /= U[i + (size_t)i * ldu];
            const double xi = x[i];
            const double* ui = U + (size_t)i * ldu;
            for (int r = 0; r < i; ++r) x[r] = std::fma(ui[r], -xi, x[r]);
        }
    }
}

// ----------------------------------------------------------------- PLU
// Panel LU with partial pivoting on columns [r0, r0+bs) (Mat's __PLU2_piv,
// LU/__PLU.h:54-90; with r0 = 0 and bs = all columns it is __PLU2,
// :22-51).  Left-looking column updates, first index attaining max |a|,
// row swaps, multiplication by the reciprocal.  Mat swaps the rows over
// columns [0, r0+bs); the swaps of the finished columns left of the panel
// (pure moves of values nothing reads again) are left to the caller.
// Returns the panel column at which a zero column stopped it (Mat's
// `break`), or -1.
int plu_panel_serial(double* A, int lda, int m, int r0, int bs, int* pos, int* piv) {
    for (int i = 0; i < bs; ++i) piv[i] = i;
    for (int c = 0; c < bs; ++c) {
        const int gc = r0 + c;
        double* col = A + (size_t)gc * lda;
        for (int i = 0; i < c; ++i) {
            const int gi = r0 + i;
            const double q = -col[gi];
            const double* li = A + (size_t)gi * lda;
            for (int r = gi + 1; r < m; ++r) col[r] = std::fma(li[r], q, col[r]);
        }
        double maxv = 0.0;
        for (int r = gc; r < m; ++r) maxv = std::max(maxv, std::fabs(col[r]));
        if (maxv == 0.0) {
            piv[c] = c;
            return c;
        }
        int j = gc;
        for (int r = gc; r < m; ++r)
            if (std::fabs(col[r]) == maxv) {
                j = r;
                break;
            }
        piv[c] = j - r0;
        if (j != gc) {
            for (int cc = r0; cc < r0 + bs; ++cc) std::swap(at(A, lda, gc, cc), at(A, lda, j, cc));
            std::swap(pos[gc], pos[j]);
        }
        const double inv = 1.0 / col[gc];
        for (int r = gc + 1; r < m; ++r) col[r] = col[r] * inv;
    }
    return -1;
}

// The same panel with its rows spread over threads.  Per column c: the rows
// above the diagonal (the U part, a serial chain through the pivots) on one
// thread, which also forms q_i = -A(r0+i, c); then every thread takes a
// chunk of the rows [r0+c, m), scales its rows of column c-1 by the previous
// pivot's reciprocal, applies fma(L(r, i), q_i, .) for i = 0..c-1 in order,
// and finds its chunk's first largest |a|; one thread picks the first
// largest over the chunks (Mat's first index) and swaps the two rows over
// the panel's columns.  Each element sees Mat's operations in Mat's order.
int plu_panel_parallel(double* A, int lda, int m, int r0, int bs, int* pos, int* piv, int nt) {
    for (int i = 0; i < bs; ++i) piv[i] = i;
    std::vector<double> q(bs), tmax(nt);
    std::vector<int> targ(nt);
    int brk = -1;
    double inv_prev = 0.0;
    SpinBarrier bar(nt);
    pool().run(nt, [&](int tid, int nth) {
        for (int c = 0; c < bs; ++c) {
            const int gc = r0 + c;
            double* col = A + (size_t)gc * lda;
            if (tid == 0) {
                for (int i = 0; i < c; ++i) {
                    const int gi = r0 + i;
                    q[i] = -col[gi];
                    const double* li = A + (size_t)gi * lda;
                    for (int r = gi + 1; r < gc; ++r) col[r] = std::fma(li[r], q[i], col[r]);
                }
            }
            bar.wait();
            int lo, hi;
            chunk(m - gc, tid, nth, lo, hi);
            lo += gc;
            hi += gc;
            if (c > 0) {
                double* pc = col - lda;
                for (int r = lo; r < hi; ++r) pc[r] = pc[r] * inv_prev;
            }
            for (int i = 0; i < c; ++i) {
                const double* li = A + (size_t)(r0 + i) * lda;
                const double qi = q[i];
                for (int r = lo; r < hi; ++r) col[r] = std::fma(li[r], qi, col[r]);
            }
            double lmax = 0.0;
            int larg = -1;
            for (int r = lo; r < hi; ++r) lmax = std::max(lmax, std::fabs(col[r]));
            for (int r = lo; r < hi; ++r)
                if (std::fabs(col[r]) == lmax) {
                    larg = r;
                    break;
                }
            tmax[tid] = lmax;
            targ[tid] = larg;
            bar.wait();
            if (tid == 0) {
                double maxv = 0.0;
                for (int t = 0; t < nth; ++t) maxv = std::max(maxv, tmax[t]);
                if (maxv == 0.0) {
                    piv[c] = c;
                    brk = c;
                } else {
                    int j = gc;
                    for (int t = 0; t < nth; ++t)
                        if (targ[t] >= 0 && tmax[t] == maxv) {
                            j = targ[t];
                            break;
                        }
                    piv[c] = j - r0;
                    if (j != gc) {
                        for (int cc = r0; cc < r0 + bs; ++cc) std::swap(at(A, lda, gc, cc), at(A, lda, j, cc));
                        std::swap(pos[gc], pos[j]);
                    }
                    inv_prev = 1.0 / col[gc];
                }
            }
            bar.wait();
            if (brk >= 0) return;
        }
        const int gl = r0 + bs - 1;
        int lo, hi;
        chunk(m - gl - 1, tid, nth, lo, hi);
        double* lc = A + (size_t)gl * lda;
        for (int r = gl + 1 + lo; r < gl + 1 + hi; ++r) lc[r] = lc[r] * inv_prev;
    });
    return brk;
}

int plu_panel(double* A, int lda, int m, int r0, int bs, int* pos, int* piv) {
    const int nt = std::min(g_threads, (m - r0) / 1024);
    if (nt < 2) return plu_panel_serial(A, lda, m, r0, bs, pos, piv);
    return plu_panel_parallel(A, lda, m, r0, bs, pos, piv, nt);
}

// Applies a panel's interchanges to columns [c0, c1) (Mat's __laswp_trailing, LU/__PLU.h:3-19).
void laswp(double* A, int lda, int r0, int kcount, int c0, int c1, const int* piv) {
    auto cols = [&](int lo, int hi) {
        for (int c = c0 + lo; c < c0 + hi; ++c) {
            double* col = A + (size_t)c * lda;
            for (int k = 0; k < kcount; ++k) {
                const int i = r0 + k, j = r0 + piv[k];
                if (i != j) std::swap(col[i], col[j]);
            }
        }
    };
    if (c1 - c0 < 256)
        cols(0, std::max(0, c1 - c0));
    else
        parallel_cols(c1 - c0, cols);
}

// In-place blocked right-looking PLU (Mat's PLU / __PLU, LU/__PLU.h:93-190).
// Returns 0, or 1 + the first column at which a zero pivot column was met.
int plu_inplace(int m, int n, double* A, int lda, int* pos) {
    for (int i = 0; i < m; ++i) pos[i] = i;
    const int s = std::min(m, n);
    int info = 0;
    std::vector<int> piv(std::max(BS_LU, n) + 1);
    if (s <= BS_LU * 1.5) {
        // __PLU2 over all columns (LU/__PLU.h:22-51): swaps every column.
        for (int c = 0; c < n && c < m; ++c) {
            double* col = A + (size_t)c * lda;
            for (int i = 0; i < c; ++i) {
                const double q = -col[i];
                const double* li = A + (size_t)i * lda;
                for (int r = i + 1; r < m; ++r) col[r] = std::fma(li[r], q, col[r]);
            }
            double maxv = 0.0;
            for (int r = c; r < m; ++r) maxv = std::max(maxv, std::fabs(col[r]));
            if (maxv == 0.0) {
                info = c + 1;
                break;
            }
            int j = c;
            for (int r = c; r < m; ++r)
                if (std::fabs(col[r]) == maxv) {
                    j = r;
                    break;
                }
            if (j != c) {
                for (int cc = 0; cc < n; ++cc) std::swap(at(A, lda, c, cc), at(A, lda, j, cc));
                std::swap(pos[c], pos[j]);
            }
            const double inv = 1.0 / col[c];
            for (int r = c + 1; r < m; ++r) col[r] = col[r] * inv;
        }
        return info;
    }
    std::vector<int> allpiv(s);  // the row each row r was swapped with (absolute)
    int r = 0;
    for (; r + BS_LU <= s; r += BS_LU) {
        const int brk = plu_panel(A, lda, m, r, BS_LU, pos, piv.data());
        if (brk >= 0 && !info) info = r + brk + 1;
        for (int k = 0; k < BS_LU; ++k) allpiv[r + k] = r + piv[k];
        laswp(A, lda, r, BS_LU, r + BS_LU, n, piv.data());
        if (r + BS_LU < s) {
            const int nt = n - (r + BS_LU);
            double* A12 = A + r + (size_t)(r + BS_LU) * lda;
            trsm_lx(BS_LU, nt, A + r + (size_t)r * lda, lda, A12, lda);
            gemm_acc(m - (r + BS_LU), nt, BS_LU, A + (r + BS_LU) + (size_t)r * lda, lda, A12, lda,
                     A + (r + BS_LU) + (size_t)(r + BS_LU) * lda, lda, true);
        }
    }
    if (r < s) {
        const int rem = s - r;
        const int brk = plu_panel(A, lda, m, r, rem, pos, piv.data());
        if (brk >= 0 && !info) info = r + brk + 1;
        for (int k = 0; k < rem; ++k) allpiv[r + k] = r + piv[k];
    }
    // Mat's interchanges of the columns left of each panel, applied at the
    // end: column c receives every later panel's swaps in order (each column
    // stays in cache while it takes them)
    const int last = r < s ? r : r - BS_LU;
    parallel_cols(std::max(0, last), [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            double* col = A + (size_t)c * lda;
            for (int k = (c / BS_LU + 1) * BS_LU; k < s; ++k)
                if (allpiv[k] != k) std::swap(col[k], col[allpiv[k]]);
        }
    });
    return info;
}

// LU without pivoting (Mat's LU / __LU / __LU2, LU/__LU.h:1-108), in place
// on a square n x n A: the PLU recipe with the diagonal as every pivot.
// __LU2 (:1-15): left-looking column updates, then the column below the
// diagonal times 1 / pivot; an exactly zero pivot stops the panel (Mat's
// `break`).  Returns 0 or 1 + the first zero-pivot column.
int lu_nopiv_panel(double* A, int lda, int m, int r0, int bs) {
    for (int c = 0; c < bs; ++c) {
        const int gc = r0 + c;
        double* col = A + (size_t)gc * lda;
        for (int i = 0; i < c; ++i) {
            const int gi = r0 + i;
            const double q = -col[gi];
            const double* li = A + (size_t)gi * lda;
            for (int r = gi + 1; r < m; ++r) col[r] = std::fma(li[r], q, col[r]);
        }
        if (col[gc] == 0.0) return c;
        const double inv = 1.0 / col[gc];
        for (int r = gc + 1; r < m; ++r) col[r] = col[r] * inv;
    }
    return -1;
}

int lu_nopiv(int n, double* A, int lda) {
    int info = 0;
    if (n <= BS_LU * 1.5) {
        const int brk = lu_nopiv_panel(A, lda, n, 0, n);
        return brk >= 0 ? brk + 1 : 0;
    }
    int r = 0;
    for (; r + BS_LU <= n; r += BS_LU) {
        const int brk = lu_nopiv_panel(A, lda, n, r, BS_LU);
        if (brk >= 0 && !info) info = r + brk + 1;
        if (r + BS_LU < n) {
            const int nt = n - (r + BS_LU);
            double* A12 = A + r + (size_t)(r + BS_LU) * lda;
            trsm_lx(BS_LU, nt, A + r + (size_t)r * lda, lda, A12, lda);
            gemm_acc(n - (r + BS_LU), nt, BS_LU, A + (r + BS_LU) + (size_t)r * lda, lda, A12, lda,
                     A + (r + BS_LU) + (size_t)(r + BS_LU) * lda, lda, true);
        }
    }
    if (r < n) {
        const int brk = lu_nopiv_panel(A, lda, n, r, n - r);
        if (brk >= 0 && !info) info = r + brk + 1;
    }
    return info;
}

// ----------------------------------------------------------------- LLT
// Unblocked Cholesky of a k x k block (Mat's __LLT2, LU/__LLT.h:3-13).
void llt2(double* L, int ldl, int k) {
    for (int j = 0; j < k; ++j) {
        const double t = 1.0 / std::sqrt(at(L, ldl, j, j));
        double* cj = L + (size_t)j * ldl;
        for (int r = j; r < k; ++r) cj[r] = cj[r] * t;
        for (int i = j + 1; i < k; ++i) {
            const double q = -at(L, ldl, i, j);
            double* ci = L + (size_t)i * ldl;
            for (int r = i; r < k; ++r) ci[r] = std::fma(cj[r], q, ci[r]);
        }
    }
}

// X(rows x k) := X * L^{-T} (Mat's __Solve_direct_XLT, LU/__LLT.h:30-40).
void trsm_xlt(int rows, int k, const double* L, int ldl, double* X, int ldx) {
    for (int j = 0; j < k; ++j) {
        double* x = X + (size_t)j * ldx;
        const double t = 1.0 / L[j + (size_t)j * ldl];
        for (int r = 0; r < rows; ++r) x[r] = x[r] * t;
        for (int kk = j + 1; kk < k; ++kk) {
            const double q = -L[kk + (size_t)j * ldl];
            double* xk = X + (size_t)kk * ldx;
            for (int r = 0; r < rows; ++r) xk[r] = std::fma(x[r], q, xk[r]);
        }
    }
}

// Blocked right-looking Cholesky (Mat's LLT / __LLT, LU/__LLT.h:94-150, 212-246).
// Reads the lower triangle of A into L, factors, zeroes the strict upper part.
int llt(int n, double* L, int ldl) {
    if (n <= 2 * BS_LLT) {
        llt2(L, ldl, n);
    } else {
        for (int j = 0; j < n; j += BS_LLT) {
            const int nb = std::min(BS_LLT, n - j);
            llt2(L + j + (size_t)j * ldl, ldl, nb);
            if (j + BS_LLT < n) {
                for (int i = j + BS_LLT; i < n; i += BS_LLT) {
                    const int mb = std::min(BS_LLT, n - i);
                    trsm_xlt(mb, BS_LLT, L + j + (size_t)j * ldl, ldl, L + i + (size_t)j * ldl, ldl);
                }
                // C(k.., i..i+m) -= L(k.., j..j+BS) * L(i..i+m, j..j+BS)^T for k >= i
                for (int i = j + BS_LLT; i < n; i += BS_LLT) {
                    const int mb = std::min(BS_LLT, n - i);
                    gemm_abt_sub(n - i, mb, BS_LLT, L + i + (size_t)j * ldl, ldl, L + i + (size_t)j * ldl, ldl,
                                 L + i + (size_t)i * ldl, ldl);
                }
            }
        }
    }
    for (int i = 0; i < n; ++i)
        for (int r = 0; r < i; ++r) at(L, ldl, r, i) = 0.0;
    for (int i = 0; i < n; ++i)
        if (!(at(L, ldl, i, i) > 0.0)) return i + 1;
    return 0;
}

// Unblocked LDL^T of a k x k block (Mat's __LDLT2, LU/__LLT.h:16-27): d_j =
// L(j,j); column j (diagonal included) times 1/d_j; then for i > j,
// q = (-L(i,j)) d_j and L(r,i) = fma(L(r,j), q, L(r,i)) for r >= i.
void ldlt2(double* L, int ldl, int k, double* d) {
    for (int j = 0; j < k; ++j) {
        d[j] = at(L, ldl, j, j);
        const double t = 1.0 / d[j];
        double* cj = L + (size_t)j * ldl;
        for (int r = j; r < k; ++r) cj[r] = cj[r] * t;
        for (int i = j + 1; i < k; ++i) {
            const double q = -at(L, ldl, i, j) * d[j];
            double* ci = L + (size_t)i * ldl;
            for (int r = i; r < k; ++r) ci[r] = std::fma(cj[r], q, ci[r]);
        }
    }
}

// Blocked LDL^T (Mat's LDLT / __LDLT, LU/__LLT.h:153-209, 249-295): as the
// Cholesky, with __Solve_direct_XDLT (:43-56: X := X L^{-T}, then each column
// times 1/d_j) below the diagonal block and the trailing update
// C -= L21 (L21 D)^T, the packed B operand holding the rounded products
// L(c, p) d_p (__pack_BT_block_d, Mul/__pack_double.h:241-282).
int ldlt(int n, double* L, int ldl, double* d) {
    if (n <= 2 * BS_LLT) {
        ldlt2(L, ldl, n, d);
    } else {
        std::vector<double> W;
        for (int j = 0; j < n; j += BS_LLT) {
            const int nb = std::min(BS_LLT, n - j);
            ldlt2(L + j + (size_t)j * ldl, ldl, nb, d + j);
            if (j + BS_LLT < n) {
                const int rows = n - j - BS_LLT;
                double* P = L + (j + BS_LLT) + (size_t)j * ldl;
                trsm_xlt(rows, nb, L + j + (size_t)j * ldl, ldl, P, ldl);
                for (int p = 0; p < nb; ++p) {
                    const double t = 1.0 / d[j + p];
                    for (int r = 0; r < rows; ++r) P[r + (size_t)p * ldl] = P[r + (size_t)p * ldl] * t;
                }
                W.assign((size_t)rows * nb, 0.0);
                for (int p = 0; p < nb; ++p)
                    for (int r = 0; r < rows; ++r) W[r + (size_t)p * rows] = P[r + (size_t)p * ldl] * d[j + p];
                for (int i = j + BS_LLT; i < n; i += BS_LLT) {
                    const int mb = std::min(BS_LLT, n - i);
                    const int off = i - (j + BS_LLT);
                    gemm_abt_sub(n - i, mb, nb, P + off, ldl, W.data() + off, rows, L + i + (size_t)i * ldl, ldl);
                }
            }
        }
    }
    for (int i = 0; i < n; ++i)
        for (int r = 0; r < i; ++r) at(L, ldl, r, i) = 0.0;
    for (int i = 0; i < n; ++i)
        if (d[i] == 0.0) return i + 1;
    return 0;
}

// ------------------------------------------------------------------ QR
// Householder panel (Mat's __QR_HouseHolder_Blocked2, QR/__Householder_Blocked.h:63-84):
// LAPACK-style v (v0 = 1 implicit, stored below the diagonal), tau = (x0+cr)/cr,
// R_rr = -cr with cr = sign(x0) ||x||.
void qr_panel(double* R, int ldr, int h, int b, double* tau, std::vector<double>& v) {
    v.resize(h);
    for (int r = 0; r < b; ++r) {
        double* w = R + r + (size_t)r * ldr;
        const int len = h - r;
        double cr = std::sqrt(dot_mat(w, w, len));
        if (cr == 0.0) {
            tau[r] = 0.0;
            continue;
        }
        if (w[0] < 0.0) cr = -cr;
        const double w0 = w[0] + cr;
        const double hr = 1.0 / w0;
        w[0] = -cr;
        for (int i = 1; i < len; ++i) w[i] = w[i] * hr;
        v[0] = 1.0;
        for (int i = 1; i < len; ++i) v[i] = w[i];
        tau[r] = w0 / cr;
        for (int c = r + 1; c < b; ++c) {
            double* col = R + r + (size_t)c * ldr;
            const double d = col[0] + dot_mat(v.data() + 1, col + 1, len - 1);
            const double q = -d * tau[r];
            for (int i = 0; i < len; ++i) col[i] = std::fma(v[i], q, col[i]);
        }
    }
}

// Upper-triangular T of the compact WY form (Mat's CalculateT, :87-103).
void qr_T(const double* V, int ldv, int h, int k, const double* tau, double* T /* k x k, ld k */) {
    std::vector<double> s(k), w(k);
    std::fill(T, T + (size_t)k * k, 0.0);
    T[0] = tau[0];
    for (int i = 1; i < k; ++i) {
        for (int l = 0; l < i; ++l) {
            const double* vl = V + (size_t)l * ldv;
            const double* vi = V + (size_t)i * ldv;
            s[l] = vl[i] + dot_generic(vl + i + 1, vi + i + 1, h - i - 1);
        }
        for (int r = 0; r < i; ++r) w[r] = 0.0;
        for (int c = 0; c < i; ++c)
            for (int r = 0; r <= c; ++r) w[r] = std::fma(T[r + (size_t)c * k], s[c], w[r]);
        for (int r = 0; r < i; ++r) T[r + (size_t)i * k] = w[r] * -tau[i];
        T[i + (size_t)i * k] = tau[i];
    }
}

// Unit-lower V (h x k) expanded into a dense copy (implicit ones, zeros above).
std::vector<double> expand_v(const double* V, int ldv, int h, int k) {
    std::vector<double> Vd((size_t)h * k, 0.0);
    for (int c = 0; c < k; ++c)
        for (int r = c; r < h; ++r) Vd[r + (size_t)c * h] = r == c ? 1.0 : V[r + (size_t)c * ldv];
    return Vd;
}

// R(h x nc) := (I - V op(T) V^T) R; op(T) = T^T for the factorization
// (…_Mul, :144-212) and T for building Q (CalculateQ, :248-333).
void apply_block_reflector(const std::vector<double>& Vd, int h, int k, const double* T, bool transT, double* R,
                           int ldr, int nc) {
    if (nc <= 0) return;
    // W = V^T R  (k x nc)
    std::vector<double> W((size_t)k * nc, 0.0), W2((size_t)k * nc, 0.0);
    parallel_cols(nc, [&](int j0, int j1) {
        for (int j = j0; j < j1; ++j)
            for (int i = 0; i < k; ++i) {
                double acc = 0.0;
                const double* vi = Vd.data() + (size_t)i * h;
                const double* rj = R + (size_t)j * ldr;
                for (int p = i; p < h; ++p) acc = std::fma(vi[p], rj[p], acc);
                W[i + (size_t)j * k] = acc;
            }
    });
    // W2 = op(T) W
    for (int j = 0; j < nc; ++j)
        for (int i = 0; i < k; ++i) {
            double acc = 0.0;
            if (transT)
                for (int p = 0; p <= i; ++p) acc = std::fma(T[p + (size_t)i * k], W[p + (size_t)j * k], acc);
            else
                for (int p = i; p < k; ++p) acc = std::fma(T[i + (size_t)p * k], W[p + (size_t)j * k], acc);
            W2[i + (size_t)j * k] = acc;
        }
    // R -= V W2
    gemm_acc(h, nc, k, Vd.data(), h, W2.data(), k, R, ldr, true);
}

// Unblocked Householder QR (Mat's __QR_HouseHolder + __HouseHolder_Q1,
// QR/__HouseHolder.h:179-208, 48-79), used when min(m,n) <= 2*BS_QR.  The
// reflectors are kept where Mat keeps them, w_r at Q + 2 m r - r^2 (length
// m - r, scaled so that w^T w = 2), and Q is accumulated backwards in place
// in the trailing square blocks of Q's storage exactly as Mat does.
void qr_unblocked(int m, int n, double* R, double* Q) {
    const int k = std::min(m, n);
    for (int r = 0; r < k; ++r) {
        double* w = Q + 2 * (size_t)m * r - (size_t)r * r;
        const int len = m - r;
        std::memcpy(w, R + r + (size_t)r * m, sizeof(double) * len);
        double cr = std::sqrt(dot_mat(w, w, len));
        if (cr == 0.0) continue;
        if (w[0] < 0.0) cr = -cr;
        w[0] += cr;
        const double hr = 1.0 / std::sqrt(cr * w[0]);
        for (int i = 0; i < len; ++i) w[i] = w[i] * hr;
        for (int c = r; c < n; ++c) {  // __ApplyHouseHolderOnTheLeft2(R, w, r, r)
            double* col = R + r + (size_t)c * m;
            const double d = -dot_mat(w, col, len);
            for (int i = 0; i < len; ++i) col[i] = std::fma(w[i], d, col[i]);
        }
    }
    // __HouseHolder_Q1(Q, k)
    int r2 = m - k;
    double* T2 = Q + (size_t)m * m - (size_t)r2 * r2;
    std::fill(T2, T2 + (size_t)r2 * r2, 0.0);
    for (int i = 0; i < r2; ++i) T2[(size_t)i * r2 + i] = 1.0;
    for (int r = k - 1; r >= 0; --r) {
        const int r1 = m - r;
        double* T1 = Q + (size_t)m * m - (size_t)r1 * r1;
        std::fill(T1 + r1, T1 + r1 + (r1 - 1), 0.0);
        double* w = T1;
        for (int i = 1; i < r1; ++i) {
            const double temp = -dot_mat(w + 1, T2 + (size_t)(i - 1) * r2, r2);
            T1[(size_t)i * r1] = w[0] * temp;
            double* dst = T1 + (size_t)i * r1 + 1;
            const double* src = T2 + (size_t)(i - 1) * r2;
            for (int e = 0; e < r2; ++e) dst[e] = std::fma(w[1 + e], temp, src[e]);  // in place, forward
        }
        const double q = -w[0];
        for (int e = 0; e < r1; ++e) w[e] = w[e] * q;
        w[0] += 1.0;
        T2 = T1;
        r2 = r1;
    }
    // Mat's unblocked path leaves R's below-diagonal entries as the reflection
    // computed them (rounding-level values), unlike the blocked path.
}

// Solve_direct_narrow's substitutions (LU/__Solve_direct.h:118-139) on the
// in-place factors a (unit L below the diagonal, U on and above it) for up
// to four right-hand sides X (n x nrhs, ld n).  Forward: for k = 0..n-2,
// x[r] = fma(L(r,k), -x[k], x[r]) for r > k; backward: for r = n-1..1,
// x[r] /= U(r,r), x[i] = fma(U(i,r), -x[r], x[i]) for i < r; x[0] /= U(0,0).
// Blocks of NB columns: the rows inside the block on one thread (the serial
// chain), the rows outside it spread over threads; each element still sees
// its updates in Mat's order.
void narrow_substitution(int n, int nrhs, const double* a, double* X) {
    constexpr int NB = 256;
    const int nt = std::min(g_threads, n / 1024);
    SpinBarrier bar(std::max(nt, 1));
    pool().run(std::max(nt, 1), [&](int tid, int nth) {
        for (int b0 = 0; b0 < n; b0 += NB) {
            const int b1 = std::min(n, b0 + NB);
            if (tid == 0)
                for (int k = b0; k < std::min(b1, n - 1); ++k) {
                    const double* lk = a + (size_t)k * n;
                    for (int j = 0; j < nrhs; ++j) {
                        double* x = X + (size_t)j * n;
                        const double q = -x[k];
                        for (int r = k + 1; r < b1; ++r) x[r] = std::fma(lk[r], q, x[r]);
                    }
                }
            bar.wait();
            int lo, hi;
            chunk(n - b1, tid, nth, lo, hi);
            lo += b1;
            hi += b1;
            for (int k = b0; k < b1 && lo < hi; ++k) {
                const double* lk = a + (size_t)k * n;
                for (int j = 0; j < nrhs; ++j) {
                    double* x = X + (size_t)j * n;
                    const double q = -x[k];
                    for (int r = lo; r < hi; ++r) x[r] = std::fma(lk[r], q, x[r]);
                }
            }
            bar.wait();
        }
        for (int b1 = n; b1 > 0; b1 -= NB) {
            const int b0 = std::max(0, b1 - NB);
            if (tid == 0)
                for (int r = b1 - 1; r >= b0; --r) {
                    const double* ur = a + (size_t)r * n;
                    for (int j = 0; j < nrhs; ++j) {
                        double* x = X + (size_t)j * n;
                        x[r] /= ur[r];
                        if (r == 0) continue;
                        const double q = -x[r];
                        for (int i = b0; i < r; ++i) x[i] = std::fma(ur[i], q, x[i]);
                    }
                }
            bar.wait();
            int lo, hi;
            chunk(b0, tid, nth, lo, hi);
            for (int r = b1 - 1; r >= b0 && lo < hi; --r) {
                const double* ur = a + (size_t)r * n;
                for (int j = 0; j < nrhs; ++j) {
                    double* x = X + (size_t)j * n;
                    const double q = -x[r];
                    for (int i = lo; i < hi; ++i) x[i] = std::fma(ur[i], q, x[i]);
                }
            }
            bar.wait();
        }
    });
}

// ------------------------------------------------------ seeded inputs
// The library's seeded matrices (mg_host_fill_*, mg_gen_svd_matrix)
// regenerated on the host: each entry depends only on (seed, index), so the
// fill is spread over threads by columns.
void host_fill(double* A, int rows, int cols, int ld, uint64_t key, double lo, double hi, bool rowmajor,
               bool normal) {
    auto fill = [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c)
            for (int r = 0; r < rows; ++r) {
                const uint64_t idx = rowmajor ? (uint64_t)r * cols + c : (uint64_t)r + (uint64_t)c * rows;
                A[r + (size_t)c * ld] = normal ? mgrng::normal_at(key, idx) : mgrng::uniform_at(key, idx, lo, hi);
            }
    };
    if ((size_t)rows * cols < (1u << 16))
        fill(0, cols);
    else
        parallel_cols(cols, fill);
}

// T (k x k, upper) of Q = H_0 ... H_{k-1} = I - V T V^T from G = V^T V, the
// forward recurrence of the block reflector (plain multiply and add, no
// contraction), as mg_gen_svd_matrix forms it on the host.
void svd_build_T(int k, const std::vector<double>& G, std::vector<double>& T) {
    T.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) {
        const double tau = 2.0 / G[i + (size_t)i * k];
        for (int r = 0; r < i; ++r) {
            double s = 0.0;
            for (int c = r; c < i; ++c) s += T[r + (size_t)c * k] * G[c + (size_t)i * k];
            T[r + (size_t)i * k] = -tau * s;
        }
        T[i + (size_t)i * k] = tau;
    }
}

}  // namespace

extern "C" {

void orc_set_threads(int n) { g_threads = std::max(1, n); }

// Mat operator* (Mul/Mul.h:204-235): C = A B, C zeroed first (Mul.h:167).
void orc_dgemm(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc) {
    for (int j = 0; j < n; ++j) std::memset(C + (size_t)j * ldc, 0, sizeof(double) * (size_t)std::max(m, 0));
    gemm_acc(m, n, k, A, lda, B, ldb, C, ldc, false);
}

void orc_host_fill_uniform(double* A, int rows, int cols, int ld, uint64_t seed, double lo, double hi,
                           int rowmajor_stream) {
    if (!A || rows <= 0 || cols <= 0) return;
    host_fill(A, rows, cols, ld, mgrng::stream_key(seed, mgrng::kSaltUniform), lo, hi, rowmajor_stream != 0, false);
}

void orc_host_fill_normal(double* A, int rows, int cols, int ld, uint64_t seed, int rowmajor_stream) {
    if (!A || rows <= 0 || cols <= 0) return;
    host_fill(A, rows, cols, ld, mgrng::stream_key(seed, mgrng::kSaltNormal), 0, 0, rowmajor_stream != 0, true);
}

// The library's mg_gen_svd_matrix on the host: A = Q1 diag(sigma) Q2,
// sigma_r = mgrng::geometric_at(r, n, sigma_min), V1, V2 (n x k) iid N(0,1)
// with seeds 2 seed + 1 and 2 seed + 2 (row-major streams), G = V^T V and T
// as above, then A := A - V (T (V^T A)) with V1 and A := A - ((A V) T) V^T
// with V2.  Every product is a fused chain in order from zero (or from A for
// the subtractions), as the GPU's FP64 GEMM computes it, so the result is
// the GPU's bit for bit.  Returns 0, or 1 for invalid arguments.
int orc_gen_svd_matrix(int n, double* A, int lda, uint64_t seed, int nrefl, double sigma_min) {
    if (n < 0 || lda < std::max(n, 1) || nrefl < 0 || (n && !A) || !(sigma_min > 0.0 && sigma_min <= 1.0)) return 1;
    if (n == 0) return 0;
    parallel_cols(n, [&](int c0, int c1) {
        for (int c = c0; c < c1; ++c) {
            double* col = A + (size_t)c * lda;
            std::fill(col, col + n, 0.0);
            col[c] = mgrng::geometric_at(c, n, sigma_min);
        }
    });
    const int k = nrefl;
    if (k == 0) return 0;
    const size_t nk = (size_t)n * k;
    std::vector<double> V(nk), Vt(nk), W(nk), W2(nk), G((size_t)k * k), T;
    for (int side = 0; side < 2; ++side) {
        orc_host_fill_normal(V.data(), n, k, n, seed * 2 + 1 + side, 1);
        for (int c = 0; c < k; ++c)
            for (int r = 0; r < n; ++r) Vt[c + (size_t)r * k] = V[r + (size_t)c * n];
        std::fill(G.begin(), G.end(), 0.0);
        gemm_acc(k, k, n, Vt.data(), k, V.data(), n, G.data(), k, false);
        svd_build_T(k, G, T);
        std::fill(W.begin(), W.end(), 0.0);
        std::fill(W2.begin(), W2.end(), 0.0);
        if (side == 0) {
            gemm_acc(k, n, n, Vt.data(), k, A, lda, W.data(), k, false);   // W = V^T A
            gemm_acc(k, n, k, T.data(), k, W.data(), k, W2.data(), k, false);  // W2 = T W
            gemm_acc(n, n, k, V.data(), n, W2.data(), k, A, lda, true);    // A -= V W2
        } else {
            gemm_acc(n, k, n, A, lda, V.data(), n, W.data(), n, false);    // W = A V
            gemm_acc(n, k, k, W.data(), n, T.data(), k, W2.data(), n, false);  // W2 = W T
            gemm_core(n, n, k, W2.data(), n, V.data(), n, true, A, lda, true);  // A -= W2 V^T
        }
    }
    return 0;
}

// In-place Mat PLU: A := L\U (unit L below the diagonal), pos as Mat returns it.
int orc_dgetrf(int m, int n, double* A, int lda, int* pos) { return plu_inplace(m, n, A, lda, pos); }

// PLU(A, pos, L, U) (LU/__PLU.h:152-190): L m x m unit lower, U m x n upper.
int orc_plu(int m, int n, const double* A, int* pos, double* L, double* U) {
    std::memcpy(U, A, sizeof(double) * (size_t)m * n);
    const int info = plu_inplace(m, n, U, m, pos);
    std::fill(L, L + (size_t)m * m, 0.0);
    const int s = std::min(m, n);
    for (int c = 0; c < s; ++c) {
        at(L, m, c, c) = 1.0;
        for (int r = c + 1; r < m; ++r) {
            at(L, m, r, c) = at(U, m, r, c);
            at(U, m, r, c) = 0.0;
        }
    }
    return info;
}

// Solve_direct(A, B) (LU/__Solve_direct.h:70-220).  For <= 4 right-hand
// sides, Mat's narrow path: in-place PLU, permute, scalar forward and back
// substitution (:112-139).  Wider: blocked substitution by the same TRSMs.
int orc_solve(int n, int nrhs, const double* A, const double* B, double* X) {
    // A is taken by value (Mat copies it); the copy and the substitutions are
    // spread over threads, each element keeping its operation sequence.
    std::unique_ptr<double[]> abuf(new double[(size_t)n * n + 1]);
    double* ad_w = abuf.get();
    parallel_cols(n, [&](int c0, int c1) {
        std::memcpy(ad_w + (size_t)c0 * n, A + (size_t)c0 * n, sizeof(double) * (size_t)n * (c1 - c0));
    });
    std::vector<int> pos(n);
    const int info = plu_inplace(n, n, ad_w, n, pos.data());
    for (int j = 0; j < nrhs; ++j)
        for (int i = 0; i < n; ++i) X[i + (size_t)j * n] = B[pos[i] + (size_t)j * n];
    const double* ad = ad_w;
    if (nrhs <= 4) {
        narrow_substitution(n, nrhs, ad, X);
    } else if (n <= BS_LU * 3 / 2) {
        // one block (:166-190)
        trsm_lx(n, nrhs, ad, n, X, n);
        trsm_ux(n, nrhs, ad, n, X, n);
    } else {
        // __Solve_direct_LU_X (:1-66): blocks of BS_LU rows; forward, each
        // block's TRSM then X(below) -= L(below, block) X(block); backward
        // from the last block, X(above) -= U(above, block) X(block).  The
        // NC / MC tiling of the products leaves each element's chain unchanged.
        for (int r = 0; r < n; r += BS_LU) {
            const int l = std::min(BS_LU, n - r);
            trsm_lx(l, nrhs, ad + r + (size_t)r * n, n, X + r, n);
            if (r + l < n) gemm_acc(n - r - l, nrhs, l, ad + (r + l) + (size_t)r * n, n, X + r, n, X + r + l, n, true);
        }
        for (int r = ((n - 1) / BS_LU) * BS_LU; r >= 0; r -= BS_LU) {
            const int l = std::min(BS_LU, n - r);
            trsm_ux(l, nrhs, ad + r + (size_t)r * n, n, X + r, n);
            if (r > 0) gemm_acc(r, nrhs, l, ad + (size_t)r * n, n, X + r, n, X, n, true);
        }
    }
    return info;
}

// LLT(A, L) (LU/__LLT.h:212-246): lower triangle of A in, L out (upper zeroed).
int orc_llt(int n, const double* A, double* L) {
    std::fill(L, L + (size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int r = c; r < n; ++r) at(L, n, r, c) = A[r + (size_t)c * n];
    return llt(n, L, n);
}

// LU(A, L, U) without pivoting (LU/__LU.h:71-108), square n: L unit lower,
// U upper.
int orc_lu(int n, const double* A, double* L, double* U) {
    std::vector<double> a(A, A + (size_t)n * n);
    const int info = lu_nopiv(n, a.data(), n);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
            const double v = a[r + (size_t)c * n];
            at(L, n, r, c) = r > c ? v : (r == c ? 1.0 : 0.0);
            at(U, n, r, c) = r <= c ? v : 0.0;
        }
    return info;
}

// LDLT(A, L, D) (LU/__LLT.h:249-295): lower triangle of A in; L (upper
// zeroed) and D = diag(d) out.
int orc_ldlt(int n, const double* A, double* L, double* D) {
    std::fill(L, L + (size_t)n * n, 0.0);
    std::fill(D, D + (size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int r = c; r < n; ++r) at(L, n, r, c) = A[r + (size_t)c * n];
    std::vector<double> d(n);
    const int info = ldlt(n, L, n, d.data());
    for (int i = 0; i < n; ++i) at(D, n, i, i) = d[i];
    return info;
}

// QR(A, Q, R, QR_Householder) (QR/QR.h:8-25): Q m x m, R m x n.
void orc_qr(int m, int n, const double* A, double* Q, double* R) {
    std::memcpy(R, A, sizeof(double) * (size_t)m * n);
    const int k = std::min(m, n);
    if (k <= 2 * BS_QR) {
        qr_unblocked(m, n, R, Q);
        return;
    }
    // Factorization (:215-245).
    std::vector<double> tau(k), v;
    std::vector<std::vector<double>> Ts;
    for (int j = 0; j < k; j += BS_QR) {
        const int b = std::min(BS_QR, k - j);
        const int h = m - j;
        double* P = R + j + (size_t)j * m;
        qr_panel(P, m, h, b, tau.data() + j, v);
        std::vector<double> T((size_t)b * b);
        qr_T(P, m, h, b, tau.data() + j, T.data());
        if (j + b < n) apply_block_reflector(expand_v(P, m, h, b), h, b, T.data(), true, P + (size_t)b * m, m,
                                             n - j - b);
        Ts.push_back(std::move(T));
    }
    // Full m x m Q, accumulated backwards (:248-333).
    std::fill(Q, Q + (size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) Q[i + (size_t)i * m] = 1.0;
    const int last = ((k - 1) / BS_QR) * BS_QR;
    for (int j = last, t = (int)Ts.size() - 1; j >= 0; j -= BS_QR, --t) {
        const int b = std::min(BS_QR, k - j);
        const int h = m - j;
        apply_block_reflector(expand_v(R + j + (size_t)j * m, m, h, b), h, b, Ts[t].data(), false,
                              Q + j, m, m);
    }
    for (int j = 0; j < n; ++j)
        for (int r = j + 1; r < m; ++r) R[r + (size_t)j * m] = 0.0;
}

// Row-wise right solves of Mat's Inv (AVX-512 __Solve_direct_XU / _XL,
// LU/__Base.h:541-662, RB = 8).  Each row x of the len x n block X is
// independent; a row in the 8-row vector part of its block (rows
// 0 .. len - len % 8 - 1) sums the eight products q_u x_u as a tree, a row in
// the scalar tail as a chain.  g++ contracts both (the intrinsics are plain
// vector arithmetic to it): the tree becomes e_u = fma(x_2u, q_2u,
// x_2u+1 q_2u+1), (e0 + e1) + (e2 + e3); the chain t = q1 x1,
// t = fma(q0, x0, t), then t = fma(q_u, x_u, t) for u = 2..7.  Both forms
// are pinned by the reference build's outputs.
static double sum8_vec(const double* q, const double* x) {
    const double e0 = std::fma(x[0], q[0], x[1] * q[1]), e1 = std::fma(x[2], q[2], x[3] * q[3]);
    const double e2 = std::fma(x[4], q[4], x[5] * q[5]), e3 = std::fma(x[6], q[6], x[7] * q[7]);
    return (e0 + e1) + (e2 + e3);
}
static double sum8_tail(const double* q, const double* x) {
    double t = q[1] * x[1];
    t = std::fma(q[0], x[0], t);
    for (int u = 2; u < 8; ++u) t = std::fma(q[u], x[u], t);
    return t;
}

// X := X U^{-1}, U unit upper n x n (diagonal not read).
static void inv_xu(int len, int n, const double* U, int ldu, double* X, int ldx) {
    const int lvec = len - len % 8;
    for (int row = 0; row < len; ++row) {
        double* x = X + row;  // x[c * ldx]
        auto xc = [&](int c) -> double& { return x[(size_t)c * ldx]; };
        int r = 0;
        for (; r + 8 <= n; r += 8) {
            for (int j = r; j < r + 8; ++j)
                for (int i = j + 1; i < r + 8; ++i) xc(i) = std::fma(xc(j), -U[j + (size_t)i * ldu], xc(i));
            double xv[8];
            for (int u = 0; u < 8; ++u) xv[u] = xc(r + u);
            for (int i = r + 8; i < n; ++i) {
                double q[8];
                for (int u = 0; u < 8; ++u) q[u] = -U[(r + u) + (size_t)i * ldu];
                xc(i) = xc(i) + (row < lvec ? sum8_vec(q, xv) : sum8_tail(q, xv));
            }
        }
        for (; r < n; ++r)
            for (int i = r + 1; i < n; ++i) xc(i) = std::fma(xc(r), -U[r + (size_t)i * ldu], xc(i));
    }
}

// X := X L^{-1}, L unit lower n x n (diagonal not read).
static void inv_xl(int len, int n, const double* L, int ldl, double* X, int ldx) {
    const int lvec = len - len % 8;
    for (int row = 0; row < len; ++row) {
        double* x = X + row;
        auto xc = [&](int c) -> double& { return x[(size_t)c * ldx]; };
        int r = n - 1;
        for (; r - 7 >= 1; r -= 8) {
            for (int j = r; j > r - 7; --j)
                for (int i = r - 7; i < j; ++i) xc(i) = std::fma(xc(j), -L[j + (size_t)i * ldl], xc(i));
            double xv[8];
            for (int u = 0; u < 8; ++u) xv[u] = xc(r - u);
            for (int i = 0; i < r - 7; ++i) {
                double q[8];
                for (int u = 0; u < 8; ++u) q[u] = -L[(r - u) + (size_t)i * ldl];
                xc(i) = xc(i) + (row < lvec ? sum8_vec(q, xv) : sum8_tail(q, xv));
            }
        }
        for (; r > 0; --r)
            for (int i = 0; i < r; ++i) xc(i) = std::fma(xc(r), -L[r + (size_t)i * ldl], xc(i));
    }
}

// Inv(A) (LU/__Inv.h:80-225): PLU; U's columns scaled by the reciprocal of
// their diagonal, X = diag(1 / u_ii); X := X U^{-1} then X := X L^{-1}
// (one block for n <= 90, else __Inv_X_LU's blocks of 60 with fused-chain
// products); columns permuted, Ainv(:, pos[i]) = X(:, i).  Returns the PLU
// zero-column index or -1.
int orc_inv(int n, const double* A, double* Ainv) {
    std::vector<double> a(A, A + (size_t)n * n), X((size_t)n * n, 0.0);
    std::vector<int> pos(n);
    const int info = plu_inplace(n, n, a.data(), n, pos.data());
    for (int i = 0; i < n; ++i) {
        const double t = 1.0 / a[i + (size_t)i * n];
        for (int j = 0; j < i; ++j) a[j + (size_t)i * n] *= t;
        X[i + (size_t)i * n] = t;
    }
    const double* ad = a.data();
    double* xd = X.data();
    if (n <= BS_LU * 3 / 2) {
        inv_xu(n, n, ad, n, xd, n);
        inv_xl(n, n, ad, n, xd, n);
    } else {
        for (int r = 0; r < n; r += BS_LU) {  // :12-44
            const int l = std::min(BS_LU, n - r);
            for (int i = 0; i <= r; i += BS_LU) {
                const int m = std::min(BS_LU, n - i);
                inv_xu(m, l, ad + r + (size_t)r * n, n, xd + i + (size_t)r * n, n);
            }
            const int rows = std::min(r + l, n);
            if (r + BS_LU < n)
                gemm_acc(rows, n - r - BS_LU, l, xd + (size_t)r * n, n, ad + r + (size_t)(r + BS_LU) * n, n,
                         xd + (size_t)(r + BS_LU) * n, n, true);
        }
        for (int r = ((n - 1) / BS_LU) * BS_LU; r >= 0; r -= BS_LU) {  // :46-77
            const int nb = std::min(BS_LU, n - r);
            for (int i = 0; i < n; i += BS_LU) {
                const int m = std::min(BS_LU, n - i);
                inv_xl(m, nb, ad + r + (size_t)r * n, n, xd + i + (size_t)r * n, n);
            }
            if (r > 0) gemm_acc(n, r, nb, xd + (size_t)r * n, n, ad + r, n, xd, n, true);
        }
    }
    for (int i = 0; i < n; ++i)
        std::memcpy(Ainv + (size_t)pos[i] * n, xd + (size_t)i * n, sizeof(double) * n);
    return info;
}

// Det(A) (LU/__Det.h:30-101): sign of the interchanges times the product of U's diagonal.
double orc_det(int n, const double* A) {
    std::vector<double> a(A, A + (size_t)n * n);
    std::vector<int> pos(n);
    plu_inplace(n, n, a.data(), n, pos.data());
    // parity of the permutation pos
    std::vector<char> seen(n, 0);
    int swaps = 0;
    for (int i = 0; i < n; ++i) {
        if (seen[i]) continue;
        int len = 0;
        for (int j = i; !seen[j]; j = pos[j]) {
            seen[j] = 1;
            ++len;
        }
        swaps += len - 1;
    }
    double ret = (swaps & 1) ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) ret = ret * a[i + (size_t)i * n];
    return ret;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Mat-8.1 snapshot: EVD_Q's Householder tridiagonalisation and the Q it forms
// (EVD/__QR.h:2-47, QR/__Householder.h:124-152).  These use the snapshot's
// own AVX-512 helpers (SIMD/__AVX512_double.h), whose dot product differs
// from Mat-8.3.1's.

// Mat-8.1's __dot (SIMD/__AVX512_double.h:111-124): one 8-lane fused
// accumulator over the full 8-blocks, the masked fused tail into lanes
// 0..rem-1 of the same accumulator, then the 8 -> 4 -> 2 -> 1 horizontal sum
// of _mm512_reduce_add_pd.
static double dot81(const double* a, const double* b, int len) {
    double acc[8] = {0};
    const int nb = len / 8;
    for (int i = 0; i < nb; ++i)
        for (int l = 0; l < 8; ++l) acc[l] = std::fma(a[i * 8 + l], b[i * 8 + l], acc[l]);
    const int rem = len - nb * 8;
    for (int l = 0; l < rem; ++l) acc[l] = std::fma(a[nb * 8 + l], b[nb * 8 + l], acc[l]);
    double h4[4], h2[2];
    for (int l = 0; l < 4; ++l) h4[l] = acc[l] + acc[l + 4];
    for (int l = 0; l < 2; ++l) h2[l] = h4[l] + h4[l + 2];
    return h2[0] + h2[1];
}

// __EVD_Q_Householder (EVD/__QR.h:2-47) on column-major storage: step m
// reduces the trailing N' = n - m matrix W (only its lower triangle is read)
// with the reflector w of its first column, w = (x + sign(x0)||x|| e0) /
// sqrt(cr (x0 + cr)), through v = W22 w (the column-wise fused chains of
// __mixed, then the dot of the rest of each column), h = v.w and the rank-2
// update W' = W22 - w v^T - v w^T + h w w^T, evaluated per column i as
// fma(w_k, fma(w_i, h, -v_i), fma(v_k, -w_i, W22_ki)) (g++ contracts
// -v[i] + w[i]*hr).  d = diagonal, e = off-diagonal (e_m = -cr), U = the
// reflectors (column m holds w_m in rows m+1..n-1).
static void tridiag81(int n, const double* A, int lda, double* d, double* e, std::vector<double>& U) {
    std::vector<double> W((size_t)n * n), Wn((size_t)n * n), v(n), w(n);
    for (int j = 0; j < n; ++j)
        for (int i = j; i < n; ++i) W[(size_t)j * n + i] = A[(size_t)j * lda + i];
    U.assign((size_t)n * n, 0.0);
    int N = n;  // leading dimension (= order) of the current trailing matrix
    for (int m = 0; m + 2 < n; ++m, --N) {
        const int nn = N - 1;
        const double temp = W[0];
        for (int k = 0; k < nn; ++k) w[k] = W[1 + k];
        double cr = std::sqrt(dot81(w.data(), w.data(), nn));
        if (w[0] < 0.0) cr = -cr;
        w[0] = w[0] + cr;
        const double hr = 1.0 / std::sqrt(cr * w[0]);
        for (int k = 0; k < nn; ++k) w[k] = w[k] * hr;
        auto Wc = [&](int r, int c) { return W[(size_t)c * N + r]; };
        for (int k = 0; k < nn; ++k) v[k] = 0.0;
        for (int i = 0; i < nn; ++i)
            for (int k = i; k < nn; ++k) v[k] = std::fma(Wc(1 + k, 1 + i), w[i], v[k]);
        for (int i = 0; i < nn; ++i)
            v[i] = v[i] + dot81(&W[(size_t)(i + 1) * N + i + 2], &w[i + 1], nn - i - 1);
        const double h = dot81(v.data(), w.data(), nn);
        for (int i = 0; i < nn; ++i) {
            const double q = std::fma(w[i], h, -v[i]);
            for (int k = i; k < nn; ++k)
                Wn[(size_t)i * nn + k] = std::fma(w[k], q, std::fma(v[k], -w[i], Wc(1 + k, 1 + i)));
        }
        std::swap(W, Wn);
        d[m] = temp;
        e[m] = -cr;
        for (int k = 0; k < nn; ++k) U[(size_t)m * n + m + 1 + k] = w[k];
    }
    if (n >= 2) {
        d[n - 2] = W[0];
        d[n - 1] = W[3];
        e[n - 2] = W[1];
    } else if (n == 1) {
        d[0] = W[0];
    }
}

// __Householder_Q2 (QR/__Householder.h:124-152): Q accumulated backwards from
// the trailing 2 x 2 identity; at level r (order t = n - r) column 0 is e0
// and column i >= 1 is (0, M_{:,i-1} + w_r (-dot(w_r, M_{:,i-1}))), M the
// previous level's (t - 1) x (t - 1) matrix.
static void form_q81(int n, const std::vector<double>& U, double* Q, int ldq) {
    if (n == 1) {
        Q[0] = 1.0;
        return;
    }
    std::vector<double> M(4, 0.0), Mn;
    M[0] = M[3] = 1.0;
    for (int r = n - 3; r >= 0; --r) {
        const int t = n - r, t2 = t - 1;
        const double* u = &U[(size_t)r * n + r + 1];
        Mn.assign((size_t)t * t, 0.0);
        Mn[0] = 1.0;
        for (int i = 1; i < t; ++i) {
            const double* mc = &M[(size_t)(i - 1) * t2];
            const double s = -dot81(u, mc, t2);
            for (int k = 0; k < t2; ++k) Mn[(size_t)i * t + 1 + k] = std::fma(u[k], s, mc[k]);
        }
        std::swap(M, Mn);
    }
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) Q[(size_t)j * ldq + i] = M[(size_t)j * n + i];
}

// One plane rotation of __EVD_Q_Givens (EVD/__QR.h:78-96 and 109-136) on the
// pair (a_i, a_i1, b_i) from the ratio t: it returns (c, s) of the rotation
// applied to Q's columns i, i+1.  `small` selects the branch whose t is
// numerator / denominator with the smaller magnitude on top of b (first
// branch: s^2 = 1/(t^2 + 1); second: c^2 = 1/(t^2 + 1)).  The reference build
// contracts t*t + 1, c2*temp + s2*temp_2 (first product), the added or
// subtracted 2*cs*b_i, and -cs*temp + cs*temp_2 + (c2 - s2)*b_i (first and
// last products).
static void rot81(double* a, double* b, int i, double t, bool first, double& c, double& s) {
    double c2, s2, cs;
    if (first) {
        s2 = 1.0 / std::fma(t, t, 1.0);
        c2 = 1.0 - s2;
        cs = t * s2;
    } else {
        c2 = 1.0 / std::fma(t, t, 1.0);
        s2 = 1.0 - c2;
        cs = t * c2;
    }
    const double temp = a[i], temp_2 = a[i + 1];
    const double cs2 = 2.0 * cs;
    a[i] = std::fma(cs2, b[i], std::fma(c2, temp, s2 * temp_2));
    a[i + 1] = std::fma(-cs2, b[i], std::fma(s2, temp, c2 * temp_2));
    b[i] = std::fma(c2 - s2, b[i], std::fma(-cs, temp, cs * temp_2));
    if (first) {
        s = std::sqrt(s2);
        c = t * s;
    } else {
        c = std::sqrt(c2);
        s = t * c;
    }
}

// __ApplyGivensOnTheRight(Q[i], Q[i+1], c, s, rows) (SIMD/__AVX512_double.h:1-20).
static void apply_rot81(double* Q, int n, int i, double c, double s) {
    double* x = Q + (size_t)i * n;
    double* y = Q + (size_t)(i + 1) * n;
    for (int r = 0; r < n; ++r) {
        const double xi = x[r], yi = y[r];
        x[r] = std::fma(xi, c, yi * s);
        y[r] = std::fma(-xi, s, yi * c);
    }
}

// __EVD_Q_Givens (EVD/__QR.h:50-142): implicit single-shift QR sweeps on the
// tridiagonal (a = diagonal, b = off-diagonal, indices m..n inclusive) with
// absolute deflation threshold eps, splitting at interior negligible b_i by
// recursion; every rotation is applied to Q's columns.  The shift is the
// eigenvalue of the trailing 2 x 2 block nearer a_n (the reference build
// evaluates c2^2 - 4 (a_{n-1} a_n - b_{n-1}^2) with both leading products
// fused).  Returns false when the sweep budget runs out.
static bool givens81(double* a, double* b, double* Q, int N, int m, int n, double eps, long long& budget) {
    while (n > m) {
        if (std::fabs(b[m]) < eps) {
            ++m;
            continue;
        }
        if (std::fabs(b[n - 1]) < eps) {
            --n;
            continue;
        }
        for (int i = m + 1; i < n - 1; ++i) {
            if (std::fabs(b[i]) < eps) {
                if (!givens81(a, b, Q, N, m, i, eps, budget)) return false;
                m = i + 1;
            }
        }
        if (--budget < 0) return false;
        double c2 = a[n - 1] + a[n];
        double s2 = std::sqrt(std::fma(c2, c2, -(std::fma(a[n - 1], a[n], -(b[n - 1] * b[n - 1])) * 4.0)));
        double t = (c2 - 2.0 * a[n] > 0) ? (c2 - s2) * 0.5 : (c2 + s2) * 0.5;
        double c, s;
        if (std::fabs(b[m]) > std::fabs(a[m] - t))
            rot81(a, b, m, (a[m] - t) / b[m], true, c, s);
        else
            rot81(a, b, m, b[m] / (a[m] - t), false, c, s);
        double B = s * b[m + 1];
        b[m + 1] = c * b[m + 1];
        apply_rot81(Q, N, m, c, s);
        for (int i = m + 1; i < n; ++i) {
            if (std::fabs(B) > std::fabs(b[i - 1]))
                rot81(a, b, i, b[i - 1] / B, true, c, s);
            else
                rot81(a, b, i, B / b[i - 1], false, c, s);
            b[i - 1] = std::fma(c, b[i - 1], s * B);
            B = s * b[i + 1];
            b[i + 1] = c * b[i + 1];
            apply_rot81(Q, N, i, c, s);
        }
    }
    return true;
}

extern "C" {

// The tridiagonalisation of EVD_Q (Mat-8.1/EVD/__QR.h:2-47, with Q formed by
// QR/__Householder.h:124-152): A symmetric n x n (lower triangle read),
// d (n), e (n - 1), Q (n x n, ld ldq) with Q^T A Q = tridiag(e, d, e).
void orc_tridiag81(int n, const double* A, int lda, double* Q, int ldq, double* d, double* e) {
    std::vector<double> U;
    tridiag81(n, A, lda, d, e, U);
    form_q81(n, U, Q, ldq);
}


// EVD_Q(A, E, Q, eps, EVD_QR) of the Mat-8.1 snapshot (EVD/EVD_Q.h:7-35 ->
// EVD/__QR.h:145-169): eigenvalues in w (E's diagonal), eigenvectors in Q's
// columns (n x n, ld n).  Returns 0, or 1 when the QR sweeps did not deflate
// within 64 n sweeps (the reference loops on).
int orc_evd_q81(int n, const double* A, double eps, double* w, double* Q) {
    std::vector<double> e((size_t)n + 1, 0.0);
    orc_tridiag81(n, A, n, Q, n, w, e.data());
    e[n > 0 ? n - 1 : 0] = 0.0;
    long long budget = 64LL * n;
    return givens81(w, e.data(), Q, n, 0, n - 1, eps, budget) ? 0 : 1;
}

}  // extern "C"
