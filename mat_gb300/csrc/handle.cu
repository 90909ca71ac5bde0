// Handle, workspace and memory utilities of the C ABI.
#include <cstdarg>
#include <cstdlib>

#include "mg_internal.cuh"

namespace mg {

mg_status_t fail(mg_handle_t h, mg_status_t s, const char* fmt, ...) {
    if (h) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(h->last_error, sizeof(h->last_error), fmt, ap);
        va_end(ap);
    }
    return s;
}

mg_status_t cuda_fail(mg_handle_t h, cudaError_t e, const char* what) {
    return fail(h, MG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

mg_status_t ensure_lookahead(mg_handle_t h) {
    if (h->la_stream) return MG_OK;
    int least = 0, greatest = 0;
    MG_CHECK_CUDA(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
    MG_CHECK_CUDA(h, cudaStreamCreateWithPriority(&h->la_stream, cudaStreamNonBlocking, least));
    for (cudaEvent_t& e : h->la_ev) MG_CHECK_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    MG_CHECK_CUDA(h, cudaStreamCreateWithPriority(&h->pp_stream, cudaStreamNonBlocking, greatest));
    for (cudaEvent_t& e : h->pp_ev) MG_CHECK_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return MG_OK;
}

mg_status_t ensure_ws(mg_handle_t h, size_t bytes) {
    if (bytes <= h->ws_bytes) return MG_OK;
    bytes = align_up(bytes + (bytes >> 3), 1 << 20);
    if (h->ws) {
        MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
        MG_CHECK_CUDA(h, cudaFree(h->ws));
        h->ws = nullptr;
        h->ws_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&h->ws, bytes);
    if (e != cudaSuccess) {
        h->ws = nullptr;
        return fail(h, MG_ERR_ALLOC, "workspace cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    h->ws_bytes = bytes;
    return MG_OK;
}

mg_status_t ensure_hws(mg_handle_t h, size_t bytes) {
    if (bytes <= h->hws_bytes) return MG_OK;
    bytes = align_up(bytes, 4096);
    if (h->hws) {
        MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
        cudaFreeHost(h->hws);
        h->hws = nullptr;
        h->hws_bytes = 0;
    }
    cudaError_t e = cudaMallocHost(&h->hws, bytes);
    if (e != cudaSuccess) {
        h->hws = nullptr;
        return fail(h, MG_ERR_ALLOC, "pinned workspace (%zu): %s", bytes, cudaGetErrorString(e));
    }
    h->hws_bytes = bytes;
    return MG_OK;
}

mg_status_t post_launch(mg_handle_t h, const char* name) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(h, MG_ERR_CUDA, "launch of %s: %s", name, cudaGetErrorString(e));
    h->launches++;
    return MG_OK;
}

static cudaEvent_t prof_event(mg_handle_t h) {
    if (!h->prof_pool.empty()) {
        cudaEvent_t e = h->prof_pool.back();
        h->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

ProfScope::ProfScope(mg_handle_t h_, const char* name, double flops_, double bytes_)
    : h(h_), flops(flops_), bytes(bytes_) {
    if (!h || !h->prof_on) return;
    if (!h->prof_only.empty() && h->prof_only != name) return;
    int idx = -1;
    for (size_t i = 0; i < h->prof.size(); ++i)
        if (h->prof[i].name == name) idx = (int)i;
    if (idx < 0) {
        h->prof.push_back({});
        h->prof.back().name = name;
        idx = (int)h->prof.size() - 1;
    }
    rec = idx;
    a = prof_event(h);
    cudaEventRecord(a, h->stream);
}

ProfScope::~ProfScope() {
    if (rec < 0 || !a) return;
    cudaEvent_t b = prof_event(h);
    cudaEventRecord(b, h->stream);
    h->prof_pending.push_back({rec, a, b, flops, bytes});
}

void prof_host(mg_handle_t h, const char* name, double ms, double count) {
    if (!h || !h->prof_on) return;
    if (!h->prof_only.empty() && h->prof_only != name) return;
    for (auto& r : h->prof)
        if (r.name == name) {
            r.ms += ms;
            r.flops += count;
            r.launches += 1;
            return;
        }
    h->prof.push_back({});
    auto& r = h->prof.back();
    r.name = name;
    r.ms = ms;
    r.flops = count;
    r.launches = 1;
}

static void prof_resolve(mg_handle_t h) {
    if (h->prof_pending.empty()) return;
    cudaStreamSynchronize(h->stream);
    for (auto& p : h->prof_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            auto& r = h->prof[p.rec];
            r.ms += ms;
            r.flops += p.flops;
            r.bytes += p.bytes;
            r.launches += 1;
        }
        h->prof_pool.push_back(p.a);
        h->prof_pool.push_back(p.b);
    }
    h->prof_pending.clear();
}

}  // namespace mg

extern "C" {

mg_status_t mg_profile_enable(mg_handle_t h, int on) {
    if (!h) return MG_ERR_ARG;
    mg::prof_resolve(h);
    h->prof_on = on != 0;
    if (on) h->prof.clear();
    return MG_OK;
}

mg_status_t mg_profile_only(mg_handle_t h, const char* name) {
    if (!h) return MG_ERR_ARG;
    h->prof_only = name ? name : "";
    return MG_OK;
}

int mg_profile_count(mg_handle_t h) {
    if (!h) return 0;
    mg::prof_resolve(h);
    return (int)h->prof.size();
}

mg_status_t mg_profile_get(mg_handle_t h, int i, const char** name, double* ms, long long* launches, double* flops,
                           double* bytes) {
    if (!h) return MG_ERR_ARG;
    mg::prof_resolve(h);
    if (i < 0 || i >= (int)h->prof.size()) return MG_ERR_ARG;
    const auto& r = h->prof[i];
    if (name) *name = r.name.c_str();
    if (ms) *ms = r.ms;
    if (launches) *launches = r.launches;
    if (flops) *flops = r.flops;
    if (bytes) *bytes = r.bytes;
    return MG_OK;
}

mg_status_t mg_handle_create(mg_handle_t* out, void* cuda_stream) {
    if (!out) return MG_ERR_ARG;
    *out = nullptr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return MG_ERR_CUDA;
    mg_handle_t h = new (std::nothrow) mg_handle_s();
    if (!h) return MG_ERR_ALLOC;
    h->stream = (cudaStream_t)cuda_stream;
    h->device = dev;
    if (cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&h->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess) {
        delete h;
        return MG_ERR_CUDA;
    }
    if (cudaMalloc(&h->status, 4096) != cudaSuccess) {
        delete h;
        return MG_ERR_ALLOC;
    }
    *out = h;
    return MG_OK;
}

mg_status_t mg_handle_destroy(mg_handle_t h) {
    if (!h) return MG_ERR_ARG;
    mg::prof_resolve(h);
    for (cudaEvent_t e : h->prof_pool) cudaEventDestroy(e);
    if (h->ws || h->hws) cudaStreamSynchronize(h->stream);
    if (h->la_stream) {
        cudaStreamSynchronize(h->la_stream);
        cudaStreamDestroy(h->la_stream);
    }
    for (cudaEvent_t e : h->la_ev)
        if (e) cudaEventDestroy(e);
    if (h->pp_stream) {
        cudaStreamSynchronize(h->pp_stream);
        cudaStreamDestroy(h->pp_stream);
    }
    for (cudaEvent_t e : h->pp_ev)
        if (e) cudaEventDestroy(e);
    if (h->ws) cudaFree(h->ws);
    for (int i = 0; i < 3; ++i)
        if (h->tcws[i]) cudaFree(h->tcws[i]);
    if (h->tcerr) cudaFree(h->tcerr);
    if (h->hws) cudaFreeHost(h->hws);
    if (h->status) cudaFree(h->status);
    delete h;
    return MG_OK;
}

mg_status_t mg_set_stream(mg_handle_t h, void* cuda_stream) {
    if (!h) return MG_ERR_ARG;
    h->stream = (cudaStream_t)cuda_stream;
    return MG_OK;
}

mg_status_t mg_synchronize(mg_handle_t h) {
    if (!h) return MG_ERR_ARG;
    MG_CHECK_CUDA(h, cudaStreamSynchronize(h->stream));
    return MG_OK;
}

const char* mg_status_string(mg_status_t s) {
    switch (s) {
        case MG_OK: return "MG_OK";
        case MG_ERR_ARG: return "MG_ERR_ARG";
        case MG_ERR_CUDA: return "MG_ERR_CUDA";
        case MG_ERR_ALLOC: return "MG_ERR_ALLOC";
        case MG_SINGULAR: return "MG_SINGULAR";
        case MG_NOT_SPD: return "MG_NOT_SPD";
        case MG_IR_STALLED: return "MG_IR_STALLED";
        case MG_FALLBACK_USED: return "MG_FALLBACK_USED";
        case MG_TIMEOUT: return "MG_TIMEOUT";
        case MG_ERR_UNSUPPORTED: return "MG_ERR_UNSUPPORTED";
        case MG_NOT_CONVERGED: return "MG_NOT_CONVERGED";
    }
    return "MG_UNKNOWN";
}

const char* mg_get_last_error(mg_handle_t h) { return h ? h->last_error : ""; }

uint64_t mg_launch_count(mg_handle_t h) { return h ? h->launches : 0; }

mg_status_t mg_device_malloc(void** out, size_t bytes) {
    if (!out) return MG_ERR_ARG;
    return cudaMalloc(out, bytes) == cudaSuccess ? MG_OK : MG_ERR_ALLOC;
}

mg_status_t mg_device_free(void* p) { return cudaFree(p) == cudaSuccess ? MG_OK : MG_ERR_CUDA; }

mg_status_t mg_host_malloc_pinned(void** out, size_t bytes) {
    if (!out) return MG_ERR_ARG;
    return cudaMallocHost(out, bytes) == cudaSuccess ? MG_OK : MG_ERR_ALLOC;
}

mg_status_t mg_host_free_pinned(void* p) { return cudaFreeHost(p) == cudaSuccess ? MG_OK : MG_ERR_CUDA; }

mg_status_t mg_memcpy(mg_handle_t h, void* dst, const void* src, size_t bytes, int kind) {
    if (!h || (bytes && (!dst || !src))) return MG_ERR_ARG;
    cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice
                     : kind == 1 ? cudaMemcpyDeviceToHost
                                 : cudaMemcpyDeviceToDevice;
    if (bytes == 0) return MG_OK;
    MG_CHECK_CUDA(h, cudaMemcpyAsync(dst, src, bytes, k, h->stream));
    return MG_OK;
}

}  // extern "C"
