// rts_batch.cpp -- batched form (rts_batch_run) and the serving loop
// (rts_server_*) of the cross-based pipeline.
//
// Batched form: the n pairs become 2n views of one view table; every stage is
// one launch over all views (k_batch.cu).  The five launches (and the reset of
// the row summaries) are captured once per batch shape into a CUDA graph; a
// later call with the same shape re-uploads only the view table (its image and
// output pointers) and replays the graph.  The tile parameters of the stages
// (rows per vertical block; one block per item, or resident blocks striding
// over the items and how many per SM) are picked per batch shape by timing the
// candidates on the first call (autotuner).
//
// Serving loop: requests are admitted in arrival order while a slot and enough
// of the server's device pool (cost-volume bytes of the request, e.g. a 40 GB
// budget) are free; admitted requests are launched as batches on a ring of
// streams, so a batch formed from requests that arrived while others were
// running overlaps with them on the device.  Completion is polled with events.
// With priority_pixels, requests of at least that many pixels form a second
// class: each runs alone on a stream above the small requests' priority (the
// older large request above the newer), no small request starts while a large
// one runs (unless it has waited 8 ms), and the small requests' launches have
// short items, so a large request's blocks are dispatched as soon as the small
// ones' retire.  Pinned host staging is kept in a cache across requests
// (pinning pages is slow, and freeing them waits for the device).
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>

#include "rts_internal.h"
#include "rts_pipe.h"
#include "rts_views.h"

namespace rts {
rts_status validate_params(rts_ctx *c, const rts_params &p, int H, int W);
}

using namespace rts;

namespace {

bool same_except_d(const rts_params &a, const rts_params &b) {
    rts_params x = a, y = b;
    x.disp_range = y.disp_range = 0;
    return memcmp(&x, &y, sizeof(rts_params)) == 0;
}

std::string shape_key(int n, const rts_pair *pairs, const rts_params *params) {
    std::string k;
    k.reserve(16 * n + sizeof(rts_params));
    k.append((const char *)&params[0], sizeof(rts_params));
    for (int i = 0; i < n; i++) {
        const int d[4] = {pairs[i].width, pairs[i].height, params[i].disp_range,
                          pairs[i].left_rgb ? 1 : 0};
        k.append((const char *)d, sizeof(d));
    }
    return k;
}

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    void *arena = nullptr;     // the arena the graph's kernels and memset address
    size_t arena_bytes = 0;
    CrossTune tune;
    uint64_t launches = 0;     // kernel launches inside the graph
};

struct GraphCache {
    std::unordered_map<std::string, GraphEntry> graphs;
    std::unordered_map<std::string, CrossTune> tunes;
    ~GraphCache() {
        for (auto &kv : graphs)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    }
};

GraphCache *cache_of(rts_ctx *c) {
    if (!c->graph_cache) c->graph_cache = new GraphCache();
    return (GraphCache *)c->graph_cache;
}

// Fills image/output pointers of the 2n views of n pairs; med (or nullptr)
// holds the median-filtered arm images, left and right of every pair.
void fill_views(ViewBatch &b, int n, const rts_pair *pairs, const rts_out *outs, int right,
                const std::vector<uint8_t *> *med) {
    for (int i = 0; i < n; i++) {
        const rts_pair &q = pairs[i];
        ViewDesc &l = b.views[right ? 2 * i : i];
        l.gref = q.left_gray; l.gtar = q.right_gray; l.cref = q.left_rgb; l.ctar = q.right_rgb;
        if (!q.left_rgb || !q.right_rgb) l.cref = l.ctar = nullptr;
        l.mref = med ? (*med)[2 * i] : nullptr;
        l.mtar = med ? (*med)[2 * i + 1] : nullptr;
        l.mirror = 0;
        l.disp = outs[i].disp_left;
        l.vol = nullptr;
        if (right) {
            ViewDesc &r = b.views[2 * i + 1];
            r.gref = q.right_gray; r.gtar = q.left_gray; r.cref = l.ctar; r.ctar = l.cref;
            r.mirror = 1;
            r.disp = outs[i].disp_right;
            r.vol = nullptr;
            l.mask = outs[i].mask;
            link_pair(&b, 2 * i, 2 * i + 1);
        }
    }
}

// Bytes of the median-filtered arm images of one pair (both images, the
// channels of its colour images, else one).
size_t median_pair_bytes(const rts_pair &q) {
    const size_t np = (size_t)q.width * q.height;
    return (np * (q.left_rgb && q.right_rgb ? 3 : 1) * 2 + 255) & ~size_t(255);
}

// Median-filters the arm images of n pairs into dst[0..n) (median_pair_bytes
// each) on the context's stream; med receives the 2n image pointers.
void median_pairs(rts_ctx *c, int k, int n, const rts_pair *pairs, uint8_t *const *dst, std::vector<uint8_t *> &med) {
    StageScope sc(c, "median");
    med.resize(2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        const rts_pair &q = pairs[i];
        const bool rgb = q.left_rgb && q.right_rgb;
        const size_t bytes = (size_t)q.width * q.height * (rgb ? 3 : 1);
        med[2 * i] = dst[i];
        med[2 * i + 1] = dst[i] + bytes;
        launch_median(c->stream, rgb ? q.left_rgb : q.left_gray, med[2 * i], q.height, q.width, rgb ? 3 : 1, k);
        launch_median(c->stream, rgb ? q.right_rgb : q.right_gray, med[2 * i + 1], q.height, q.width, rgb ? 3 : 1, k);
    }
    count_launch(c, 2 * n);
}

void view_dims(int n, const rts_pair *pairs, const rts_params *params, int right, std::vector<int> &W,
               std::vector<int> &H, std::vector<int> &D) {
    const int nv = right ? 2 * n : n;
    W.resize(nv);
    H.resize(nv);
    D.resize(nv);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < (right ? 2 : 1); k++) {
            const int v = right ? 2 * i + k : i;
            W[v] = pairs[i].width;
            H[v] = pairs[i].height;
            D[v] = params[i].disp_range;
        }
}

// Candidate tiles of the autotuner.
// (strip rows of the vertical kernel, row-segment blocks per SM, persistent)
const CrossTune kTuneCandidates[] = {{4096, 8, 0}, {256, 8, 0}, {96, 8, 0}, {4096, 8, 1}, {256, 8, 1}, {4096, 6, 1}};

}  // namespace

extern "C" {

void rts_graph_cache_free(rts_ctx *c) {
    if (c && c->graph_cache) {
        delete (GraphCache *)c->graph_cache;
        c->graph_cache = nullptr;
    }
}

rts_status rts_batch_run(rts_ctx *ctx, int n, const rts_pair *pairs, const rts_params *params, rts_out *outs) {
    if (!ctx || n < 0 || (n > 0 && (!pairs || !params || !outs))) return RTS_ERR_INVALID_ARG;
    if (n == 0) return RTS_OK;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    rts_ctx *c = ctx;
    if (cudaSetDevice(c->device) != cudaSuccess) return set_error(c, RTS_ERR_CUDA, "cudaSetDevice failed");
    bool batched = params[0].aggr == RTS_AGGR_CROSS && cross_fused_supported(params[0]) && cross_record_costs(params[0]);
    for (int i = 0; i < n && batched; i++) {
        RTS_TRY(validate_params(c, params[i], pairs[i].height, pairs[i].width));
        batched = same_except_d(params[0], params[i]) && cross_fused_supported(params[i]) &&
                  (pairs[i].left_rgb != nullptr) == (pairs[0].left_rgb != nullptr);
    }
    if (!batched) {
        // other configurations: one pipeline run per pair, on the same stream
        for (int i = 0; i < n; i++) RTS_TRY(rts_pipeline_run(c, RTS_DEVICE, &pairs[i], &params[i], &outs[i]));
        return RTS_OK;
    }
    return batch_views_run(c, n, pairs, params, outs);
}

}  // extern "C"

// The batched cross-based pipeline on DEVICE buffers: one view table, autotuned
// tiles, one captured graph per batch shape.  Callers have validated the pairs.
rts_status rts::batch_views_run(rts_ctx *c, int n, const rts_pair *pairs, const rts_params *params, rts_out *outs) {
    for (int i = 0; i < n; i++)
        if (!pairs[i].left_gray || !pairs[i].right_gray || !outs[i].disp_left ||
            (params[0].right_view && (!outs[i].disp_right || !outs[i].mask)))
            return set_error(c, RTS_ERR_INVALID_ARG, "null image or output in the batch");
    const rts_params &p = params[0];
    const int right = p.right_view ? 1 : 0;
    const int nv = right ? 2 * n : n;
    std::vector<int> W, H, D;
    view_dims(n, pairs, params, right, W, H, D);
    // segment storage: exact u16 for integer costs, else by the form; half = 2-byte layout
    const int segk = cross_seg_kind(p, *std::max_element(W.begin(), W.end())), half = segk != 0;
    GraphCache *gc = cache_of(c);
    std::string key = shape_key(n, pairs, params);
    const bool forced = c->force_tune[0] > 0;
    if (forced) key.append((const char *)c->force_tune, sizeof(c->force_tune));
    const size_t bytes = views_bytes(W.data(), H.data(), D.data(), nv, half);
    void *arena;
    RTS_TRY(scratch(c, SL_BATCH0, bytes, &arena));
    // the tables the kernels read must hold this lambda pair before any replay
    RTS_TRY(cross_tables(c, p));
    int gray = 1;  // records hold the gray byte as colour only when no pair has colour images
    for (int i = 0; i < n; i++)
        if (pairs[i].left_rgb && pairs[i].right_rgb) gray = 0;
    // arms on median-filtered images: filtered ahead of the stage launches (and of the graph)
    std::vector<uint8_t *> med;
    if (p.median_ksize) {
        std::vector<uint8_t *> dst(n);
        size_t mb = 0;
        for (int i = 0; i < n; i++) mb += median_pair_bytes(pairs[i]);
        void *mv;
        RTS_TRY(scratch(c, SL_V_MED, mb, &mv));
        mb = 0;
        for (int i = 0; i < n; i++) {
            dst[i] = (uint8_t *)mv + mb;
            mb += median_pair_bytes(pairs[i]);
        }
        median_pairs(c, p.median_ksize, n, pairs, dst.data(), med);
    }
    ViewBatch b;
    plan_views_at(arena, W.data(), H.data(), D.data(), nv, half, &b);
    fill_views(b, n, pairs, outs, right, p.median_ksize ? &med : nullptr);
    // autotune once per shape: time every candidate on this batch
    auto tit = gc->tunes.find(key);
    if (tit == gc->tunes.end() && forced) {
        CrossTune ft;
        ft.vert_rows = c->force_tune[0];
        ft.grid_mult = c->force_tune[1];
        ft.persistent = c->force_tune[2];
        tit = gc->tunes.emplace(key, ft).first;
    }
    if (tit == gc->tunes.end()) {
        const bool timing = c->timing;
        c->timing = false;
        CrossTune best = kTuneCandidates[0];
        float best_ms = 1e30f;
        cudaEvent_t e0, e1;
        RTS_CU(c, cudaEventCreate(&e0));
        RTS_CU(c, cudaEventCreate(&e1));
        for (const CrossTune &cand : kTuneCandidates) {
            ViewTable t;
            RTS_TRY(upload_views(c, b, cand, nullptr, &t));
            // one untimed run (first launches of a kernel carry set-up costs), then
            // the faster of two timed runs
            for (int rep = 0; rep < 3; rep++) {
                RTS_CU(c, cudaEventRecord(e0, c->stream));
                RTS_TRY(launch_cross_views(c, p, t, segk, 0, gray, b.max_d, cand, b.row_last_all, b.row_last_count));
                RTS_CU(c, cudaEventRecord(e1, c->stream));
                RTS_CU(c, cudaEventSynchronize(e1));
                float ms = 0;
                RTS_CU(c, cudaEventElapsedTime(&ms, e0, e1));
                if (rep > 0 && ms < best_ms) {
                    best_ms = ms;
                    best = cand;
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        c->timing = timing;
        tit = gc->tunes.emplace(key, best).first;
    }
    const CrossTune tune = tit->second;
    ViewTable t;
    // a pageable upload: the host table may be reused as soon as the copy call returns
    RTS_TRY(upload_views(c, b, tune, nullptr, &t));
    if (c->timing) {
        // stage timing wants an event pair around every kernel: launch directly
        return launch_cross_views(c, p, t, segk, 0, gray, b.max_d, tune, b.row_last_all, b.row_last_count);
    }
    GraphEntry &g = gc->graphs[key];
    if (g.exec && (g.arena != arena || g.arena_bytes != bytes)) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    if (!g.exec) {
        // capture the stage launches; the view table is read from device memory,
        // so later calls only re-upload it before the replay
        const bool timing = c->timing;
        c->timing = false;
        const uint64_t l0 = c->launches.load();
        cudaGraph_t graph;
        RTS_CU(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        rts_status st = launch_cross_views(c, p, t, segk, 0, gray, b.max_d, tune, b.row_last_all, b.row_last_count);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
        c->timing = timing;
        if (st != RTS_OK) return st;
        RTS_CU(c, ce);
        ce = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        RTS_CU(c, ce);
        g.arena = arena;
        g.arena_bytes = bytes;
        g.tune = tune;
        g.launches = c->launches.load() - l0;
        c->launches.fetch_sub(g.launches);  // counted on every replay instead
    }
    {
        StageScope sc(c, "batch_graph");
        RTS_CU(c, cudaGraphLaunch(g.exec, c->stream));
        count_launch(c, (int)g.launches);
    }
    return RTS_OK;
}

// ===========================================================================
// serving loop

namespace {

using Clock = std::chrono::steady_clock;

// first-fit allocator over one device pool (the server's HBM budget)
struct Pool {
    unsigned char *base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    size_t used = 0;
    bool init(size_t bytes) {
        if (cudaMalloc(&base, bytes) != cudaSuccess) {
            cudaGetLastError();
            base = nullptr;
            return false;
        }
        size = bytes;
        free_[0] = bytes;
        return true;
    }
    void *alloc(size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                const size_t off = it->first, len = it->second;
                free_.erase(it);
                if (len > bytes) free_[off + bytes] = len - bytes;
                used += bytes;
                return base + off;
            }
        }
        return nullptr;
    }
    void release(void *p, size_t bytes) {
        if (!p) return;
        bytes = (bytes + 255) & ~size_t(255);
        size_t off = (unsigned char *)p - base;
        used -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    ~Pool() {
        if (base) cudaFree(base);
    }
};

// Pinned host staging kept across requests: pinning and unpinning pages is far
// slower than a request's copies (and freeing pinned memory waits for the
// device), so released blocks go to a free list by size and are handed out
// again; beyond `cap` cached bytes a released block is freed.
struct HostCache {
    std::multimap<size_t, unsigned char *> free_;       // block size -> block
    std::unordered_map<unsigned char *, size_t> size_;  // every live or cached block
    size_t cached = 0, cap = size_t(4) << 30;
    unsigned char *get(size_t bytes) {
        bytes = (bytes + 65535) & ~size_t(65535);
        auto it = free_.lower_bound(bytes);
        if (it != free_.end() && it->first <= 2 * bytes) {
            unsigned char *p = it->second;
            cached -= it->first;
            free_.erase(it);
            return p;
        }
        unsigned char *p = nullptr;
        if (cudaHostAlloc((void **)&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        size_[p] = bytes;
        return p;
    }
    void put(unsigned char *p) {
        if (!p) return;
        const size_t bytes = size_[p];
        if (cached + bytes > cap) {
            size_.erase(p);
            cudaFreeHost(p);
            return;
        }
        free_.emplace(bytes, p);
        cached += bytes;
    }
    ~HostCache() {
        for (auto &kv : size_) cudaFreeHost(kv.first);
    }
};

enum ReqState { RQ_PENDING, RQ_RUNNING, RQ_DONE, RQ_CANCELLED, RQ_FAILED };

struct Request {
    uint64_t ticket;
    rts_pair pair;
    rts_params params;
    rts_out out;               // caller's host buffers
    unsigned char *h_in = nullptr;  // pinned copy of the inputs: gray L, gray R, (rgb L, rgb R);
                                    // then, in the same staging block, h_out
    unsigned char *h_out = nullptr; // pinned outputs: disp L, disp R, mask
    size_t in_bytes = 0, out_bytes = 0;
    bool direct_out = false;   // the caller's output buffers are pinned: the device writes them directly
    void *d_mem = nullptr;     // device: inputs + outputs
    size_t d_bytes = 0;
    int state = RQ_PENDING;
    int batch = -1;
    double t_submit = 0, t_start = 0, t_done = 0;
};

struct Batch {
    std::vector<uint64_t> tickets;
    void *arena = nullptr;
    size_t arena_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool active = false;
    bool high = false;  // on a high-priority stream (large requests, launched alone)
    int prio = 0;       // the stream's priority (lower numbers are served first)
};

}  // namespace

struct rts_server {
    rts_ctx *ctx = nullptr;
    rts_server_config cfg{};
    Pool pool;
    std::vector<cudaStream_t> streams;
    std::vector<Batch> batches;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::deque<uint64_t> queue;
    // recently cancelled tickets whose entries are gone (off the device): wait and
    // poll still report RTS_ERR_CANCELLED for them; the oldest are forgotten past
    // kCancelMemory
    std::unordered_set<uint64_t> cancelled;
    std::deque<uint64_t> cancelled_order;
    uint64_t next_ticket = 1;
    int inflight = 0;
    int next_stream = 0;
    rts_params base_params{};
    bool have_params = false;
    HostCache staging;
    Clock::time_point t0 = Clock::now();
    std::mutex mu;
    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

namespace {

// device bytes of a request: inputs, outputs, then its median-filtered arm images
size_t request_device_bytes(const Request &r) {
    const size_t np = (size_t)r.pair.width * r.pair.height;
    return ((r.in_bytes + 255) & ~size_t(255)) + ((3 * np + 255) & ~size_t(255)) +
           (r.params.median_ksize ? median_pair_bytes(r.pair) : 0);
}

constexpr size_t kCancelMemory = 4096;

// Drops a cancelled request that is off the device and out of the queue; its
// ticket is remembered as cancelled.
void drop_cancelled(rts_server *s, uint64_t ticket) {
    s->reqs.erase(ticket);
    if (s->cancelled.insert(ticket).second) {
        s->cancelled_order.push_back(ticket);
        if (s->cancelled_order.size() > kCancelMemory) {
            s->cancelled.erase(s->cancelled_order.front());
            s->cancelled_order.pop_front();
        }
    }
}

void finish_batch(rts_server *s, Batch &bt) {
    for (uint64_t tk : bt.tickets) {
        auto it = s->reqs.find(tk);
        if (it == s->reqs.end()) continue;
        Request &r = *it->second;
        const size_t np = (size_t)r.pair.width * r.pair.height;
        if (r.state == RQ_RUNNING) {
            if (!r.direct_out) {
                memcpy(r.out.disp_left, r.h_out, np);
                if (r.params.right_view) {
                    memcpy(r.out.disp_right, r.h_out + np, np);
                    memcpy(r.out.mask, r.h_out + 2 * np, np);
                }
            }
            r.state = RQ_DONE;
        }
        r.t_done = s->now_ms();
        s->pool.release(r.d_mem, r.d_bytes);
        r.d_mem = nullptr;
        // the device is done with the staging and the result is delivered
        s->staging.put(r.h_in);
        r.h_in = r.h_out = nullptr;
        s->inflight--;
        if (r.state == RQ_CANCELLED) drop_cancelled(s, tk);  // cancelled while running: nothing to deliver
    }
    s->pool.release(bt.arena, bt.arena_bytes);
    bt.arena = nullptr;
    bt.tickets.clear();
    bt.active = false;
}

bool is_large(const rts_server *s, const Request &r) {
    return s->cfg.priority_pixels > 0 && (long long)r.pair.width * r.pair.height >= s->cfg.priority_pixels;
}

// requests the admission looks past while small ones are held
constexpr size_t kLookahead = 256;
// a small request that has waited this long starts even while a large one runs
// (no starvation under a steady stream of large requests)
constexpr double kHoldMs = 8.0;

bool large_running(const rts_server *s) {
    for (const Batch &b : s->batches)
        if (b.high && b.active) return true;
    return false;
}

// A free stream of the given class; -1 if none.  Small requests take the ring
// round robin.  The large class's streams form a ladder of priorities: a new
// large request takes the greatest free priority below that of every large
// request still running, so the oldest one keeps the SMs it needs and finishes
// in its own time, rather than every concurrent one being slowed alike (FIFO
// within the class instead of processor sharing).
int free_slot(const rts_server *s, bool high) {
    const int nb = (int)s->batches.size();
    if (!high) {
        for (int k = 0; k < nb; k++) {
            const int j = (s->next_stream + k) % nb;
            if (!s->batches[j].active && !s->batches[j].high) return j;
        }
        return -1;
    }
    bool any = false;
    int floor_prio = 0;  // the lowest priority (largest number) of the running large requests
    for (const Batch &b : s->batches)
        if (b.high && b.active) {
            floor_prio = any ? std::max(floor_prio, b.prio) : b.prio;
            any = true;
        }
    int below = -1, lowest = -1;
    for (int j = 0; j < nb; j++) {
        const Batch &b = s->batches[j];
        if (!b.high || b.active) continue;
        if ((!any || b.prio > floor_prio) && (below < 0 || b.prio < s->batches[below].prio)) below = j;
        if (lowest < 0 || b.prio > s->batches[lowest].prio) lowest = j;
    }
    return below >= 0 ? below : lowest;
}

// Launches the requests in `ids` as one batch on a free stream of their class.
rts_status launch_batch(rts_server *s, std::vector<Request *> &ids) {
    rts_ctx *c = s->ctx;
    const int slot = free_slot(s, is_large(s, *ids[0]));
    if (slot < 0) return RTS_ERR_BUSY;
    Batch &bt = s->batches[slot];
    const int n = (int)ids.size();
    const rts_params &p = s->base_params;
    const int right = p.right_view ? 1 : 0;
    std::vector<rts_pair> pairs(n);
    std::vector<rts_params> params(n);
    std::vector<rts_out> outs(n);
    for (int i = 0; i < n; i++) {
        Request &r = *ids[i];
        const size_t np = (size_t)r.pair.width * r.pair.height;
        unsigned char *d = (unsigned char *)r.d_mem;
        unsigned char *dout = d + ((r.in_bytes + 255) & ~size_t(255));
        pairs[i] = r.pair;
        pairs[i].left_gray = d;
        pairs[i].right_gray = d + np;
        pairs[i].left_rgb = r.pair.left_rgb ? d + 2 * np : nullptr;
        pairs[i].right_rgb = r.pair.right_rgb ? d + 5 * np : nullptr;
        pairs[i].left_lab = pairs[i].right_lab = nullptr;
        params[i] = r.params;
        outs[i] = rts_out{dout, dout + np, dout + 2 * np, nullptr};
    }
    std::vector<int> W, H, D;
    view_dims(n, pairs.data(), params.data(), right, W, H, D);
    const int nv = right ? 2 * n : n;
    const int segk = cross_seg_kind(p, *std::max_element(W.begin(), W.end())), half = segk != 0;
    int gray = 1;
    for (int i = 0; i < n; i++)
        if (pairs[i].left_rgb && pairs[i].right_rgb) gray = 0;
    bt.arena_bytes = views_bytes(W.data(), H.data(), D.data(), nv, half);
    bt.arena = s->pool.alloc(bt.arena_bytes);
    if (!bt.arena) return RTS_ERR_BUSY;
    cudaStream_t saved = c->stream;
    c->stream = s->streams[slot];
    rts_status st = RTS_OK;
    for (int i = 0; i < n && st == RTS_OK; i++) {
        Request &r = *ids[i];
        if (cudaMemcpyAsync(r.d_mem, r.h_in, r.in_bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            st = set_error(c, RTS_ERR_CUDA, "server H2D copy failed");
    }
    std::vector<uint8_t *> med;
    if (st == RTS_OK && p.median_ksize) {
        std::vector<uint8_t *> dst(n);
        for (int i = 0; i < n; i++) {
            const size_t np = (size_t)pairs[i].width * pairs[i].height;
            dst[i] = outs[i].disp_left + ((3 * np + 255) & ~size_t(255));
        }
        median_pairs(c, p.median_ksize, n, pairs.data(), dst.data(), med);
    }
    ViewBatch b;
    if (st == RTS_OK) {
        plan_views_at(bt.arena, W.data(), H.data(), D.data(), nv, half, &b);
        fill_views(b, n, pairs.data(), outs.data(), right, p.median_ksize ? &med : nullptr);
        ViewTable t;
        CrossTune tune;
        // one block per work item (the default): the blocks of a large request take
        // the SMs as the small requests' retire, and a block that starts late owns
        // no share of the items fixed at launch; the small requests' items are short
        if (s->cfg.priority_pixels > 0 && !bt.high) tune.vert_rows = 256;
        st = upload_views(c, b, tune, nullptr, &t);
        if (st == RTS_OK) st = launch_cross_views(c, p, t, segk, 0, gray, b.max_d, tune, b.row_last_all, b.row_last_count);
    }
    for (int i = 0; i < n && st == RTS_OK; i++) {
        Request &r = *ids[i];
        const size_t np = (size_t)r.pair.width * r.pair.height;
        bool ok;
        if (r.direct_out) {
            ok = cudaMemcpyAsync(r.out.disp_left, outs[i].disp_left, np, cudaMemcpyDeviceToHost, c->stream) ==
                     cudaSuccess &&
                 (!r.params.right_view ||
                  (cudaMemcpyAsync(r.out.disp_right, outs[i].disp_right, np, cudaMemcpyDeviceToHost, c->stream) ==
                       cudaSuccess &&
                   cudaMemcpyAsync(r.out.mask, outs[i].mask, np, cudaMemcpyDeviceToHost, c->stream) == cudaSuccess));
        } else {
            ok = cudaMemcpyAsync(r.h_out, outs[i].disp_left, r.out_bytes, cudaMemcpyDeviceToHost, c->stream) ==
                 cudaSuccess;
        }
        if (!ok) st = set_error(c, RTS_ERR_CUDA, "server D2H copy failed");
    }
    if (st == RTS_OK && cudaEventRecord(bt.done, c->stream) != cudaSuccess) st = RTS_ERR_CUDA;
    c->stream = saved;
    if (st != RTS_OK) {
        s->pool.release(bt.arena, bt.arena_bytes);
        bt.arena = nullptr;
        return st;
    }
    const double t = s->now_ms();
    for (Request *r : ids) {
        r->state = RQ_RUNNING;
        r->batch = slot;
        r->t_start = t;
        bt.tickets.push_back(r->ticket);
    }
    bt.active = true;
    bt.stream = s->streams[slot];
    s->next_stream = (slot + 1) % (int)s->batches.size();
    return RTS_OK;
}

rts_status progress_locked(rts_server *s) {
    // completions
    for (Batch &bt : s->batches) {
        if (!bt.active) continue;
        const cudaError_t q = cudaEventQuery(bt.done);
        if (q == cudaSuccess) finish_batch(s, bt);
        else if (q != cudaErrorNotReady) return cuda_check(s->ctx, q, "server batch");
    }
    // admission in arrival order while a stream of the request's class, a slot and
    // device memory are free; a large request (priority_pixels) goes alone.  While
    // a large request runs, the small ones wait (their blocks would share the SMs
    // with it), up to kHoldMs for the oldest, and a large one behind them may go
    // first.
    for (;;) {
        while (!s->queue.empty() && s->reqs[s->queue.front()]->state == RQ_CANCELLED) s->queue.pop_front();
        if (s->queue.empty()) return RTS_OK;
        size_t pos = 0;
        if (large_running(s) && s->now_ms() - s->reqs[s->queue.front()]->t_submit < kHoldMs) {
            const size_t look = std::min(s->queue.size(), kLookahead);
            while (pos < look && (s->reqs[s->queue[pos]]->state == RQ_CANCELLED ||
                                  !is_large(s, *s->reqs[s->queue[pos]])))
                pos++;
            if (pos == look) return RTS_OK;
        }
        const bool high = is_large(s, *s->reqs[s->queue[pos]]);
        if (free_slot(s, high) < 0) return RTS_OK;
        const int max_batch = high ? 1 : s->cfg.max_batch;
        std::vector<Request *> batch;
        size_t batch_bytes = 0;
        while (pos < s->queue.size() && (int)batch.size() < max_batch && s->inflight < s->cfg.max_inflight) {
            Request &r = *s->reqs[s->queue[pos]];
            if (r.state == RQ_CANCELLED) {
                s->queue.erase(s->queue.begin() + pos);
                continue;
            }
            if (is_large(s, r) != high) break;  // the next request is of the other class
            // the request's own buffers plus its share of the batch scratch
            int Wv[2] = {r.pair.width, r.pair.width}, Hv[2] = {r.pair.height, r.pair.height},
                Dv[2] = {r.params.disp_range, r.params.disp_range};
            const size_t need_scratch = views_bytes(Wv, Hv, Dv, r.params.right_view ? 2 : 1,
                                                    s->base_params.precision == RTS_PREC_F16);
            const size_t need = request_device_bytes(r);
            if (s->pool.used + batch_bytes + need + need_scratch + 65536 > s->pool.size) break;  // wait for memory
            r.d_bytes = need;
            r.d_mem = s->pool.alloc(need);
            if (!r.d_mem) break;
            batch_bytes += need_scratch;
            s->queue.erase(s->queue.begin() + pos);
            s->inflight++;
            batch.push_back(&r);
        }
        if (batch.empty()) return RTS_OK;
        rts_status st = launch_batch(s, batch);
        if (st != RTS_OK) {
            // put the requests back where they were in the queue
            for (auto it = batch.rbegin(); it != batch.rend(); ++it) {
                s->pool.release((*it)->d_mem, (*it)->d_bytes);
                (*it)->d_mem = nullptr;
                s->inflight--;
                s->queue.insert(s->queue.begin() + pos, (*it)->ticket);
            }
            return st == RTS_ERR_BUSY ? RTS_OK : st;
        }
    }
}

}  // namespace

extern "C" {

rts_status rts_server_create(rts_server **out, rts_ctx *ctx, const rts_server_config *cfg) {
    if (!out || !ctx || !cfg || cfg->hbm_budget == 0 || cfg->max_inflight <= 0 || cfg->max_batch <= 0)
        return RTS_ERR_INVALID_ARG;
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return RTS_ERR_CUDA;
    auto *s = new rts_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    if (!s->pool.init(cfg->hbm_budget)) {
        delete s;
        return set_error(ctx, RTS_ERR_OOM, "cannot reserve the server's device pool");
    }
    // three streams at the least priority; with priority_pixels, up to four more
    // for the large requests at the priorities above it, greatest first (their
    // blocks are dispatched before the small requests', the older large
    // request's before the newer's; with a single level above the least, two
    // streams share it)
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
        delete s;
        return RTS_ERR_CUDA;
    }
    const int levels = least - greatest;  // priorities above the least
    const int nlow = 3, nhigh = cfg->priority_pixels > 0 ? (levels >= 2 ? std::min(levels, 4) : 2) : 0;
    s->streams.resize(nlow + nhigh);
    s->batches.resize(nlow + nhigh);
    for (int i = 0; i < nlow + nhigh; i++) {
        Batch &b = s->batches[i];
        b.high = i >= nlow;
        b.prio = !b.high ? least : levels >= 2 ? greatest + (i - nlow) : greatest;
        if (cudaStreamCreateWithPriority(&s->streams[i], cudaStreamNonBlocking, b.prio) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->batches[i].done, cudaEventDisableTiming) != cudaSuccess) {
            rts_server_destroy(s);
            return RTS_ERR_CUDA;
        }
    }
    *out = s;
    return RTS_OK;
}

void rts_server_destroy(rts_server *s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    for (auto st : s->streams)
        if (st) cudaStreamSynchronize(st);
    for (auto &b : s->batches)
        if (b.done) cudaEventDestroy(b.done);
    for (auto st : s->streams)
        if (st) cudaStreamDestroy(st);
    delete s;
}

rts_status rts_server_submit(rts_server *s, const rts_pair *pair, const rts_params *params, rts_out *out,
                             uint64_t *ticket) {
    if (!s || !pair || !params || !out || !ticket) return RTS_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    rts_ctx *c = s->ctx;
    RTS_TRY(validate_params(c, *params, pair->height, pair->width));
    if (params->aggr != RTS_AGGR_CROSS || !cross_fused_supported(*params) || !cross_record_costs(*params))
        return set_error(c, RTS_ERR_INVALID_ARG, "the serving loop runs the fused cross-based pipeline");
    if (!s->have_params) {
        s->base_params = *params;
        s->have_params = true;
    } else if (!same_except_d(s->base_params, *params)) {
        return set_error(c, RTS_ERR_INVALID_ARG, "requests of one server share all parameters but disp_range");
    }
    if (!pair->left_gray || !pair->right_gray || !out->disp_left || (params->right_view && (!out->disp_right || !out->mask)))
        return set_error(c, RTS_ERR_INVALID_ARG, "null image or output");
    auto r = std::make_unique<Request>();
    r->ticket = s->next_ticket++;
    r->pair = *pair;
    r->params = *params;
    r->out = *out;
    const size_t np = (size_t)pair->width * pair->height;
    const bool rgb = pair->left_rgb && pair->right_rgb;
    r->pair.left_rgb = rgb ? pair->left_rgb : nullptr;
    r->pair.right_rgb = rgb ? pair->right_rgb : nullptr;
    r->in_bytes = np * (rgb ? 8 : 2);
    r->out_bytes = np * 3;
    // pinned (page-locked) output buffers are written by the device directly
    auto pinned = [](const void *q) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return a.type == cudaMemoryTypeHost;
    };
    r->direct_out = pinned(out->disp_left) && (!params->right_view || (pinned(out->disp_right) && pinned(out->mask)));
    // admission control also covers requests that could never fit
    int Wv[2] = {pair->width, pair->width}, Hv[2] = {pair->height, pair->height},
        Dv[2] = {params->disp_range, params->disp_range};
    if (request_device_bytes(*r) + views_bytes(Wv, Hv, Dv, params->right_view ? 2 : 1,
                                               params->precision == RTS_PREC_F16) > s->pool.size)
        return set_error(c, RTS_ERR_BUSY, "request larger than the server's HBM budget");
    r->h_in = s->staging.get(((r->in_bytes + 255) & ~size_t(255)) + r->out_bytes);
    if (!r->h_in) return set_error(c, RTS_ERR_OOM, "pinned host memory");
    r->h_out = r->h_in + ((r->in_bytes + 255) & ~size_t(255));
    memcpy(r->h_in, pair->left_gray, np);
    memcpy(r->h_in + np, pair->right_gray, np);
    if (rgb) {
        memcpy(r->h_in + 2 * np, pair->left_rgb, 3 * np);
        memcpy(r->h_in + 5 * np, pair->right_rgb, 3 * np);
    }
    r->t_submit = s->now_ms();
    *ticket = r->ticket;
    s->queue.push_back(r->ticket);
    s->reqs.emplace(r->ticket, std::move(r));
    return progress_locked(s);
}

rts_status rts_server_progress(rts_server *s) {
    if (!s) return RTS_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    if (cudaSetDevice(s->ctx->device) != cudaSuccess) return RTS_ERR_CUDA;
    return progress_locked(s);
}

int rts_server_poll(rts_server *s, uint64_t ticket) {
    if (!s) return -(int)RTS_ERR_INVALID_ARG;
    rts_status st = rts_server_progress(s);
    if (st != RTS_OK) return -(int)st;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return s->cancelled.count(ticket) ? -(int)RTS_ERR_CANCELLED : -(int)RTS_ERR_INVALID_ARG;
    switch (it->second->state) {
    case RQ_DONE: return 1;
    case RQ_CANCELLED: return -(int)RTS_ERR_CANCELLED;
    case RQ_FAILED: return -(int)RTS_ERR_CUDA;
    }
    return 0;
}

rts_status rts_server_wait(rts_server *s, uint64_t ticket, double timeout_ms, rts_request_stats *stats) {
    if (!s) return RTS_ERR_INVALID_ARG;
    const double t_end = s->now_ms() + timeout_ms;
    for (;;) {
        const int r = rts_server_poll(s, ticket);
        if (r == -(int)RTS_ERR_CANCELLED) return RTS_ERR_CANCELLED;  // the entry goes when it leaves the device
        if (r < 0) return (rts_status)(-r);
        if (r == 1) break;
        if (s->now_ms() > t_end) return RTS_ERR_TIMEOUT;
    }
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    Request &r = *it->second;
    if (stats) *stats = rts_request_stats{r.t_submit, r.t_start, r.t_done};
    s->reqs.erase(it);
    return RTS_OK;
}

long rts_server_tracked(rts_server *s) {
    if (!s) return -1;
    std::lock_guard<std::mutex> g(s->mu);
    return (long)s->reqs.size();
}

rts_status rts_server_cancel(rts_server *s, uint64_t ticket) {
    if (!s) return RTS_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return RTS_ERR_INVALID_ARG;
    Request &r = *it->second;
    if (r.state == RQ_PENDING) {
        // never admitted: out of the queue and forgotten now
        s->staging.put(r.h_in);
        r.h_in = r.h_out = nullptr;
        auto q = std::find(s->queue.begin(), s->queue.end(), ticket);
        if (q != s->queue.end()) s->queue.erase(q);
        drop_cancelled(s, ticket);
        return RTS_OK;
    }
    if (r.state == RQ_RUNNING) {
        r.state = RQ_CANCELLED;  // the batch finishes on the device; the result is not delivered
        return RTS_OK;
    }
    return RTS_ERR_INVALID_ARG;
}

}  // extern "C"
