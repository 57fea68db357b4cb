// rts_ctx.cpp -- context, scratch arena, host/device staging, host-computed
// lookup tables and stage timing for rtstereo_gb300.
#include <math.h>
#include <string.h>

#include <cstdio>

#include "rts_internal.h"

namespace rts {

rts_status set_error(rts_ctx *c, rts_status s, const std::string &msg) {
    if (c) c->last_error = msg;
    return s;
}

rts_status cuda_check(rts_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return RTS_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_error(c, RTS_ERR_OOM, m);
    }
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorInvalidDevice)
        return set_error(c, RTS_ERR_UNSUPPORTED, m);
    return set_error(c, RTS_ERR_CUDA, m);
}

rts_status dev_alloc(rts_ctx *c, size_t bytes, void **out) {
    *out = nullptr;
    if (bytes == 0) bytes = 256;
    if (c->budget && c->used + bytes > c->budget)
        return set_error(c, RTS_ERR_OOM, "HBM budget of the context exceeded (" + std::to_string(c->used + bytes) +
                                             " > " + std::to_string(c->budget) + " bytes)");
    cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_check(c, e, "cudaMalloc");
    }
    c->used += bytes;
    return RTS_OK;
}

void dev_free(rts_ctx *c, void *p, size_t bytes) {
    if (!p) return;
    cudaFree(p);
    c->used -= bytes;
}

rts_status scratch(rts_ctx *c, int slot, size_t bytes, void **out) {
    DevBuf &b = c->slots[slot];
    if (b.bytes < bytes) {
        // round up so that slightly growing shapes do not reallocate every call
        size_t want = bytes + bytes / 8 + 4096;
        want = (want + 4095) & ~size_t(4095);
        if (b.ptr) {
            RTS_CU(c, cudaStreamSynchronize(c->stream));
            dev_free(c, b.ptr, b.bytes);
            b.ptr = nullptr;
            b.bytes = 0;
        }
        rts_status s = dev_alloc(c, want, &b.ptr);
        if (s != RTS_OK) {
            // retry at the exact size before giving up
            s = dev_alloc(c, bytes, &b.ptr);
            if (s != RTS_OK) return s;
            want = bytes;
        }
        b.bytes = want;
    }
    *out = b.ptr;
    return RTS_OK;
}

rts_status stage_in(rts_ctx *c, rts_mem m, int slot, const void *src, size_t bytes, const void **dev) {
    if (!src) return set_error(c, RTS_ERR_INVALID_ARG, "null input pointer");
    if (m == RTS_DEVICE) {
        *dev = src;
        return RTS_OK;
    }
    void *d;
    RTS_TRY(scratch(c, slot, bytes, &d));
    RTS_CU(c, cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, c->stream));
    *dev = d;
    return RTS_OK;
}

rts_status stage_out(rts_ctx *c, rts_mem m, int slot, void *dst, size_t bytes, void **dev) {
    if (!dst) return set_error(c, RTS_ERR_INVALID_ARG, "null output pointer");
    if (m == RTS_DEVICE) {
        *dev = dst;
        return RTS_OK;
    }
    return scratch(c, slot, bytes, dev);
}

rts_status stage_inout(rts_ctx *c, rts_mem m, int slot, void *buf, size_t bytes, void **dev) {
    const void *d;
    RTS_TRY(stage_in(c, m, slot, buf, bytes, &d));
    *dev = const_cast<void *>(d);
    return RTS_OK;
}

rts_status finish_out(rts_ctx *c, rts_mem m, void *dst, const void *dev, size_t bytes) {
    if (m == RTS_DEVICE || dst == dev) return RTS_OK;
    RTS_CU(c, cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    return RTS_OK;
}

rts_status finish(rts_ctx *c, rts_mem m) {
    if (m == RTS_DEVICE) return RTS_OK;
    RTS_CU(c, cudaStreamSynchronize(c->stream));
    return RTS_OK;
}

void count_launch(rts_ctx *c, int n) { c->launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

rts_status check_launch(rts_ctx *c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_check(c, e, what);
    return RTS_OK;
}

static void drain_stage(StageTimer &t) {
    for (auto &ev : t.pending) {
        float ms = 0;
        if (cudaEventSynchronize(ev.second) == cudaSuccess && cudaEventElapsedTime(&ms, ev.first, ev.second) == cudaSuccess)
            t.total_ms += ms;
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
    }
    t.pending.clear();
}

StageScope::StageScope(rts_ctx *c_, const char *name) : c(c_), idx(-1) {
    if (!c->timing) return;
    for (size_t i = 0; i < c->stages.size(); i++)
        if (c->stages[i].name == name) idx = (int)i;
    if (idx < 0) {
        StageTimer st;
        st.name = name;
        c->stages.push_back(st);
        idx = (int)c->stages.size() - 1;
    }
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        idx = -1;
        return;
    }
    cudaEventRecord(e0, c->stream);
}

StageScope::~StageScope() {
    if (idx < 0) return;
    cudaEventRecord(e1, c->stream);
    StageTimer &t = c->stages[idx];
    t.launches++;
    t.pending.emplace_back(e0, e1);
    if (t.pending.size() > 256) drain_stage(t);
}

// ---- host tables ------------------------------------------------------------

void host_prox_weight(float *pw, float gamma_p, int rad) {
    // seq/AdaptiveWeightAggregation.cpp:11-18 in float with glibc sqrtf/expf
    int k = 0;
    for (int dy = -rad; dy <= rad; dy++)
        for (int dx = -rad; dx <= rad; dx++) {
            float r = sqrtf((float)(dy * dy + dx * dx));
            pw[k++] = expf(-r / gamma_p);
        }
}

rts_status combine_luts(rts_ctx *c, float lambda1, float lambda2, const float **l1, const float **l2) {
    void *d1, *d2;
    RTS_TRY(scratch(c, SL_LUT0, kCombineLut * sizeof(float), &d1));
    RTS_TRY(scratch(c, SL_LUT1, kCombineLut * sizeof(float), &d2));
    float lam[2] = {lambda1, lambda2};
    void *dst[2] = {d1, d2};
    for (int i = 0; i < 2; i++) {
        if (c->lut_key[i].a == lam[i] && c->lut_key[i].n == kCombineLut) continue;
        std::vector<float> t(kCombineLut);
        // seq/CombineCost.cpp:21-22: 1 - exp(-cost/lambda) on floats (glibc expf)
        for (int v = 0; v < kCombineLut; v++) t[v] = 1 - expf(-(float)v / lam[i]);
        RTS_CU(c, cudaMemcpyAsync(dst[i], t.data(), kCombineLut * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        RTS_CU(c, cudaStreamSynchronize(c->stream));
        c->lut_key[i].a = lam[i];
        c->lut_key[i].n = kCombineLut;
    }
    *l1 = (const float *)d1;
    *l2 = (const float *)d2;
    return RTS_OK;
}

rts_status recip_table(rts_ctx *c, const float **r) {
    void *d;
    RTS_TRY(scratch(c, SL_RCP, (kRecipMax + 1) * sizeof(float), &d));
    if (!c->rcp_ready) {
        std::vector<float> tab(kRecipMax + 1);
        tab[0] = 0.f;
        for (int i = 1; i <= kRecipMax; i++) tab[i] = 1.0f / (float)i;
        RTS_CU(c, cudaMemcpyAsync(d, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        RTS_CU(c, cudaStreamSynchronize(c->stream));
        c->rcp_ready = true;
    }
    *r = (const float *)d;
    return RTS_OK;
}

rts_status lab_weight_lut(rts_ctx *c, float gamma_s, const float **g) {
    void *d;
    size_t n = (size_t)kLabDist2Max + 1;
    RTS_TRY(scratch(c, SL_LUTW, n * sizeof(float), &d));
    if (c->lutw_gamma != gamma_s) {
        std::vector<float> t(n);
        // seq/AdaptiveWeightAggregation.cpp:19-24,63: colour distance sqrtf of an
        // exactly representable integer, then expf(-dist/gamma_s)
        for (size_t i = 0; i < n; i++) {
            float dist = sqrtf((float)i);
            t[i] = expf(-dist / gamma_s);
        }
        RTS_CU(c, cudaMemcpyAsync(d, t.data(), n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        RTS_CU(c, cudaStreamSynchronize(c->stream));
        c->lutw_gamma = gamma_s;
    }
    *g = (const float *)d;
    return RTS_OK;
}

rts_status prox_weights(rts_ctx *c, float gamma_p, int rad, const float **pw) {
    int area = (2 * rad + 1) * (2 * rad + 1);
    void *d;
    RTS_TRY(scratch(c, SL_PW, area * sizeof(float), &d));
    if (c->pw_gamma != gamma_p || c->pw_rad != rad) {
        std::vector<float> t(area);
        host_prox_weight(t.data(), gamma_p, rad);
        RTS_CU(c, cudaMemcpyAsync(d, t.data(), area * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        RTS_CU(c, cudaStreamSynchronize(c->stream));
        c->pw_gamma = gamma_p;
        c->pw_rad = rad;
    }
    *pw = (const float *)d;
    return RTS_OK;
}

}  // namespace rts

using namespace rts;

extern "C" {

const char *rts_status_string(rts_status s) {
    switch (s) {
    case RTS_OK: return "ok";
    case RTS_ERR_INVALID_ARG: return "invalid argument";
    case RTS_ERR_OOM: return "out of device memory or over the HBM budget";
    case RTS_ERR_CUDA: return "CUDA error";
    case RTS_ERR_TIMEOUT: return "timeout";
    case RTS_ERR_UNSUPPORTED: return "unsupported (no usable CUDA device)";
    case RTS_ERR_BUSY: return "busy";
    case RTS_ERR_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

rts_status rts_ctx_create(rts_ctx **out, int device, size_t hbm_budget) {
    if (!out) return RTS_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return RTS_ERR_UNSUPPORTED;
    }
    if (device < 0 || device >= n) return RTS_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return RTS_ERR_CUDA;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return RTS_ERR_CUDA;
    if (prop.major < 10) return RTS_ERR_UNSUPPORTED;  // built for sm_103a only
    rts_ctx *c = new rts_ctx();
    c->device = device;
    c->budget = hbm_budget;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return RTS_ERR_CUDA;
    }
    c->stream = c->own_stream;
    *out = c;
    return RTS_OK;
}

void rts_graph_cache_free(rts_ctx *c);  // rts_pipeline.cpp

void rts_ctx_destroy(rts_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    rts_graph_cache_free(c);
    for (auto &t : c->stages) {
        for (auto &ev : t.pending) {
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
    }
    for (auto &b : c->slots)
        if (b.ptr) cudaFree(b.ptr);
    for (auto &b : c->extra)
        if (b.ptr) cudaFree(b.ptr);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

rts_status rts_ctx_set_stream(rts_ctx *c, void *s) {
    if (!c) return RTS_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> g(c->mu);
    c->stream = s ? (cudaStream_t)s : c->own_stream;
    return RTS_OK;
}

void *rts_ctx_stream(rts_ctx *c) { return c ? (void *)c->stream : nullptr; }

rts_status rts_ctx_synchronize(rts_ctx *c) {
    if (!c) return RTS_ERR_INVALID_ARG;
    RTS_CU(c, cudaStreamSynchronize(c->stream));
    return RTS_OK;
}

size_t rts_ctx_bytes_in_use(const rts_ctx *c) { return c ? c->used : 0; }

const char *rts_ctx_last_error(const rts_ctx *c) { return c ? c->last_error.c_str() : "null context"; }

uint64_t rts_ctx_kernel_launches(const rts_ctx *c) { return c ? c->launches.load() : 0; }

rts_status rts_ctx_force_cross_tune(rts_ctx *c, int vert_rows, int grid_mult, int persistent) {
    if (!c || vert_rows < 0 || (vert_rows > 0 && (grid_mult < 1 || (persistent != 0 && persistent != 1))))
        return RTS_ERR_INVALID_ARG;
    c->force_tune[0] = vert_rows;
    c->force_tune[1] = grid_mult;
    c->force_tune[2] = persistent;
    return RTS_OK;
}

uint64_t rts_ctx_tma_timeouts(const rts_ctx *c) {
    if (!c || cudaSetDevice(c->device) != cudaSuccess) return 0;
    return box_tma_timeouts() + aw_tma_timeouts();
}

rts_status rts_ctx_enable_stage_timing(rts_ctx *c, int enable) {
    if (!c) return RTS_ERR_INVALID_ARG;
    c->timing = enable != 0;
    return RTS_OK;
}

int rts_ctx_stage_times(rts_ctx *c, const char **names, uint64_t *launches, double *total_ms, int max) {
    if (!c) return 0;
    int n = (int)c->stages.size();
    for (int i = 0; i < n && i < max; i++) {
        drain_stage(c->stages[i]);
        if (names) names[i] = c->stages[i].name.c_str();
        if (launches) launches[i] = c->stages[i].launches;
        if (total_ms) total_ms[i] = c->stages[i].total_ms;
    }
    return n;
}

void rts_ctx_reset_stage_times(rts_ctx *c) {
    if (!c) return;
    for (auto &t : c->stages) {
        drain_stage(t);
        t.launches = 0;
        t.total_ms = 0;
    }
}

}  // extern "C"
