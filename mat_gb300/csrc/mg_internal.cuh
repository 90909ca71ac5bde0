// Internal definitions shared by the libmatgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mat_gpu.h"

struct mg_handle_s {
    cudaStream_t stream = nullptr;
    int device = 0;
    int num_sms = 0;
    int max_smem_optin = 0;
    // Device workspace, grown on demand (cudaMalloc) and reused across calls.
    void* ws = nullptr;
    size_t ws_bytes = 0;
    // Small device area for status words (info / error flags) that must not
    // overlap the caller-visible workspace.
    int* status = nullptr;
    // Split operands of FP32 GEMMs run on the tensor cores: one area per
    // stream a factorization issues GEMMs on (the handle's stream, the
    // look-ahead side streams), and their error words.
    void* tcws[3] = {nullptr, nullptr, nullptr};
    size_t tcws_bytes[3] = {0, 0, 0};
    int* tcerr = nullptr;
    // Pinned host workspace (status words read back by info-reporting calls).
    void* hws = nullptr;
    size_t hws_bytes = 0;
    uint64_t launches = 0;
    // Cluster size of the FP32 cluster panel (0: not probed yet, -1: unavailable).
    int panel_cluster = 0;
    // Look-ahead LU: low-priority side stream (far trailing updates) and two
    // ordering events.
    cudaStream_t la_stream = nullptr;
    cudaEvent_t la_ev[2] = {nullptr, nullptr};
    // Side stream (highest priority) for panels and the work that follows a
    // panel, running beside a far trailing update, and its two ordering
    // events.
    cudaStream_t pp_stream = nullptr;
    cudaEvent_t pp_ev[2] = {nullptr, nullptr};
    char last_error[512] = {0};
    // Optional per-phase timing with CUDA events on the handle's stream.
    struct ProfRec {
        std::string name;
        double ms = 0, flops = 0, bytes = 0;
        long long launches = 0;
    };
    struct ProfPending {
        int rec;
        cudaEvent_t a, b;
        double flops, bytes;
    };
    bool prof_on = false;
    std::string prof_only;  // when not empty, only scopes of this name are timed
    std::vector<ProfRec> prof;
    std::vector<ProfPending> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
};

namespace mg {

// Records a message on the handle and returns the status.
mg_status_t fail(mg_handle_t h, mg_status_t s, const char* fmt, ...);

// Translates a CUDA error into MG_ERR_CUDA with a message.
mg_status_t cuda_fail(mg_handle_t h, cudaError_t e, const char* what);

// Grows the device workspace to at least `bytes` (synchronises when it grows).
mg_status_t ensure_ws(mg_handle_t h, size_t bytes);
mg_status_t ensure_hws(mg_handle_t h, size_t bytes);

// Checks the last launch on the handle's stream; counts it.
mg_status_t post_launch(mg_handle_t h, const char* name);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Times the launches enqueued during its lifetime under `name` when the
// handle's profiler is on (events recorded on the handle's stream); records
// the algorithmic flops / bytes of that work for roofline reporting.
// A host-timed phase in the profile (ms of host time; `count` is added to
// the record's flops field, e.g. a number of items processed).
void prof_host(mg_handle_t h, const char* name, double ms, double count);

struct ProfScope {
    mg_handle_t h;
    int rec = -1;
    cudaEvent_t a = nullptr;
    double flops, bytes;
    ProfScope(mg_handle_t h_, const char* name, double flops_ = 0, double bytes_ = 0);
    ~ProfScope();
};

// Internal GEMM launcher (no argument checking), used by the factorizations.
// Computes C = alpha*op(A)*op(B) + beta*C.  `tri` = 0 full, 1 = only tiles
// that intersect the lower triangle of C (row >= col - tile), used by the
// Cholesky trailing update.
mg_status_t dgemm_launch(mg_handle_t h, int transA, int transB, int m, int n, int k,
                         double alpha, const double* A, int lda, const double* B, int ldb,
                         double beta, double* C, int ldc, int tri);

// In-place FP64 Mat PLU and narrow solve (lu.cu).
mg_status_t dgetrf_impl(mg_handle_t h, int m, int n, double* A, int lda, int* pos, int* info_out);
// X := U^{-1} X in FP64 for an fp32 upper triangle (lu.cu).
mg_status_t upper_solve_f32_factors(mg_handle_t h, int n, int nrhs, const float* U, int ldu, double* X, int ldx);
// Mixed FP32 Householder QR (qr_mixed.cu): workspace bytes, the factorization
// (tau in FP64, T blocks of 128 x 128 fp32), and X := R^{-1} Q^T B in FP64
// (square A) with the same workspace.
size_t qr_mixed_ws_bytes(int m, int n, int num_sms);
mg_status_t sgeqrf_mixed(mg_handle_t h, int m, int n, float* A, int lda, double* tau, float* T, void* ws, int* err);
// X (fp32, n x nrhs <= 8, ld ldx) := Q^T X in fp32 with the factors of
// sgeqrf_mixed (m = n); ws as for qr_solve_f32_factors; err receives
// MG_TIMEOUT if a grid barrier of the (cooperative) kernel gave up.
mg_status_t qr_apply_qt_f32(mg_handle_t h, int n, int nrhs, const float* A, int lda, const float* T, float* X, int ldx,
                            void* ws, int* err);
mg_status_t qr_solve_f32_factors(mg_handle_t h, int n, int nrhs, const float* A, int lda, const float* T,
                                 const double* B, int ldb, double* X, int ldx, void* ws);
// X := (P^T L U)^{-1} B in FP64 for the mixed LU's fp32 in-place factors (lu.cu).
mg_status_t lu_solve_f32_factors(mg_handle_t h, int n, int nrhs, const float* LU, int lda, const int* pos,
                                 const double* B, int ldb, double* X, int ldx);
mg_status_t dgetrs_impl(mg_handle_t h, int n, int nrhs, const double* LU, int lda, const int* pos,
                        const double* B, int ldb, double* X, int ldx);
// Device workspace dgetrf_impl uses at the start of h->ws (callers place
// their own buffers after it).
size_t dgetrf_ws_bytes(int num_sms);
// Inverse from in-place PLU factors (inv.cu); LU's upper part is rescaled.
mg_status_t dinv_from_lu(mg_handle_t h, int n, double* LU, const int* pos, double* X, double* Ainv, int ldinv);

// Cholesky (chol.cu).
mg_status_t dpotrf_impl(mg_handle_t h, int n, double* L, int ldl, int* info_out);
mg_status_t dldlt_impl(mg_handle_t h, int n, double* L, int ldl, double* d, int* info_out);
template <typename T>
mg_status_t potrf_impl(mg_handle_t h, int n, T* L, int ldl, int* info_out);  // double, float
template <typename T>
mg_status_t chol_lower_solve(mg_handle_t h, int n, int nrhs, const T* L, int ldl, T* X, int ldx);
template <typename T>
mg_status_t chol_lower_t_solve(mg_handle_t h, int n, int nrhs, const T* L, int ldl, T* X, int ldx);

// FP32 SIMT GEMM (sgemm.cu), the same interface as dgemm_launch.
mg_status_t sgemm_launch(mg_handle_t h, int transA, int transB, int m, int n, int k, float alpha, const float* A,
                         int lda, const float* B, int ldb, float beta, float* C, int ldc, int tri);
// GEMM of the element type: FP64 DMMA kernel, or the FP32 SIMT kernel.
inline mg_status_t gemm_of(mg_handle_t h, int ta, int tb, int m, int n, int k, double alpha, const double* A,
                           int lda, const double* B, int ldb, double beta, double* C, int ldc, int tri) {
    return dgemm_launch(h, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
}
// The FP32 GEMM of the factorizations and adjoints: large products (k >= 32,
// m n k >= 2^27) run on the tensor cores as split-BF16 products (3 terms,
// lower-order products first, fp32 accumulation; the whole m x n block is
// computed when tri is set, callers read its lower part only), the rest on
// the SIMT FP32 kernel.
mg_status_t sgemm_auto(mg_handle_t h, int ta, int tb, int m, int n, int k, float alpha, const float* A, int lda,
                       const float* B, int ldb, float beta, float* C, int ldc, int tri);
// Sticky error word of those tensor-core GEMMs (MG_TIMEOUT after a bounded wait gave up), or 0.
mg_status_t tc_sgemm_error(mg_handle_t h, int* err_out);
inline mg_status_t gemm_of(mg_handle_t h, int ta, int tb, int m, int n, int k, float alpha, const float* A, int lda,
                           const float* B, int ldb, float beta, float* C, int ldc, int tri) {
    return sgemm_auto(h, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
}

// Split-BF16 tensor-core GEMM pieces (gemm_bf16x.cu).
size_t bf16x_split_bytes(int rows, int K, int np);
template <typename TIN>
mg_status_t bf16x_split(mg_handle_t h, bool a_side, const TIN* X, int ldx, int rows_or_cols, int K, int np,
                        void* out);
// a_term / b_term: elements between the split terms of A / B (0: M*Kp /
// N*Kp, i.e. a whole split operand; larger when the operand is a row or
// column window of a bigger split).  max_ctas > 0 caps the persistent grid.
// stream_c: C passes through L2 once (evict-first policy); false when C is
// read again soon (the next panel's columns).  two_pass: accumulate every
// lower-order product over K before the leading one (a second pass over K
// for A_0 B_0; about 6x less accumulation error, one third more operand
// loads).  lower (M == N): only the tiles that meet C's lower triangle
// (row >= column) are computed; tiles on the diagonal are computed whole.
// red_epi (used when beta == 1, C is 16-byte aligned and ldc a multiple of
// 4): the epilogue adds alpha * A B into C by TMA reductions from shared
// memory instead of loading C into registers; faster for a C that streams
// through HBM, but its L2 traffic slowed a latency-bound kernel running
// beside it (the LU's panel beside its far update).  ksplit > 1 (needs
// beta == 1 and the red_epi conditions): K is cut into ksplit slices, each
// work item one tile over one slice, every slice's product added into C.
mg_status_t bf16x_gemm_presplit(mg_handle_t h, int np, int M, int N, int K, float alpha, const void* Asplit,
                                const void* Bsplit, float beta, float* C, int ldc, int* err, size_t a_term = 0,
                                size_t b_term = 0, int max_ctas = 0, bool stream_c = true, bool two_pass = false,
                                bool lower = false, bool red_epi = false, int ksplit = 1);
// X (rows x 64, ld ldx) := X G (G: 64 x 64, column-major, ld 64) in FP32,
// the np split terms of the result as an operand with K = 64
// (bf16x_split_bytes(rows, 64, np)), and with ntop > 0 the FP32 update
// C (rows x ntop, ld ldx) -= X Xt^T, Xt (64 x 64, ld 64) holding the first
// ntop rows of the result.
mg_status_t bf16x_xlt_split64(mg_handle_t h, const float* G, float* X, int ldx, int rows, int np, void* out,
                              const float* xtop, int ntop, float* C);
// K rounded up to the split GEMM's K step (elements per row of a split term).
int bf16x_kpad(int K);
// A12 (w x nt, ld lda) := L11^{-1} A12 with L11 (w x w, ld lda) unit lower,
// w <= 128, in FP32; out receives U12's np split terms as a B operand
// (bf16x_split_bytes(nt, w, np)).
mg_status_t bf16x_trsm_split(mg_handle_t h, const float* L11, int lda, float* A12, int nt, int w, int np, void* out);

// FP32 panel on one thread-block cluster (panel_f32.cu): rows it can take
// (0 if unavailable), and the launch (piv relative to r0; pos updated).
int panel_cluster_rows(mg_handle_t h);
// tourn: tournament pivoting (one pivot agreement per 16-column sub-panel,
// CALU's TSLU over the cluster's CTAs) instead of partial pivoting.
mg_status_t sgetf2_cluster(mg_handle_t h, float* A, int lda, int m, int r0, int w, int* pos, int* piv, int* info,
                           int* err, bool tourn = false);

// FP32 LU with split-BF16 trailing updates (lu.cu).  splitA and splitA2
// each hold bf16x_split_bytes(n, nb, nterms) (the L21 split of alternate
// steps), splitB the same.
size_t sgetrf_xchg_bytes(int num_sms);
mg_status_t sgetrf_mixed(mg_handle_t h, int n, float* A, int lda, int* pos, int nb, int nterms, void* xchg,
                         void* splitA, void* splitA2, void* splitB, int* gemm_err, int* info_out,
                         bool tourn = false);
// FP32 Cholesky with split-BF16 trailing updates for the mixed SPD solve, and
// the rewrite of its factor as the packed LU of the same matrix (chol.cu).
// split: bf16x_split_bytes(n, 64, nterms); gblk: 2 x 64 x 64 floats.
mg_status_t spotrf_mixed(mg_handle_t h, int n, float* L, int ldl, int nterms, void* split, float* gblk,
                         int* gemm_err, int* info_out);
mg_status_t chol_to_lu_f32(mg_handle_t h, int n, float* A, int lda, float* dscratch);
// Side stream and events of the look-ahead LU (created once per handle).
mg_status_t ensure_lookahead(mg_handle_t h);

// Runs the enclosed launches on another stream of the handle (the profiler
// records on whatever h->stream is at the time).
struct OnStream {
    mg_handle_t h;
    cudaStream_t saved;
    OnStream(mg_handle_t h_, cudaStream_t s) : h(h_), saved(h_->stream) { h->stream = s; }
    ~OnStream() { h->stream = saved; }
};


}  // namespace mg

#define MG_CHECK_CUDA(h, call)                                   \
    do {                                                         \
        cudaError_t _e = (call);                                 \
        if (_e != cudaSuccess) return mg::cuda_fail(h, _e, #call); \
    } while (0)

#define MG_TRY(call)                                  \
    do {                                              \
        mg_status_t _s = (call);                      \
        if (_s != MG_OK) return _s;                   \
    } while (0)
