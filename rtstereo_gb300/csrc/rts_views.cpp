// rts_views.cpp -- host planning of view tables for the cross-based pipeline.
#include <string.h>

#include "rts_views.h"

namespace rts {

static size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

size_t views_bytes(const int *W, const int *H, const int *D, int n, int half) {
    size_t bytes = 0, rl = 0;
    for (int i = 0; i < n; i++) {
        const size_t np = (size_t)W[i] * H[i], ne = np * D[i];
        bytes += align256(np * 32) + align256(np * 16) + align256(ne * (half ? 2 : 4)) + align256(np * 2);
        rl += H[i];
    }
    bytes += align256(rl * 4);
    // the view table and the stage offsets
    bytes += align256(sizeof(ViewDesc) * n) + align256(sizeof(int) * ST_COUNT * (n + 1));
    return bytes;
}

void plan_views_at(void *arena, const int *W, const int *H, const int *D, int n, int half, ViewBatch *b) {
    b->views.assign(n, ViewDesc{});
    b->off.assign((size_t)ST_COUNT * (n + 1), 0);
    b->max_d = 0;
    unsigned char *a = (unsigned char *)arena;
    size_t pos = 0, rl = 0;
    for (int i = 0; i < n; i++) {
        const size_t np = (size_t)W[i] * H[i], ne = np * D[i];
        ViewDesc &v = b->views[i];
        v.W = W[i];
        v.H = H[i];
        v.D = D[i];
        v.partner = -1;
        v.prep = 1;
        v.rref = (uint4 *)(a + pos);
        v.rtar = v.rref + np;
        pos += align256(np * 32);
        v.aref = (uint2 *)(a + pos);
        v.atar = v.aref + np;
        pos += align256(np * 16);
        v.seg = a + pos;
        pos += align256(ne * (half ? 2 : 4));
        v.raw = (uint16_t *)(a + pos);
        pos += align256(np * 2);
        rl += H[i];
        if (D[i] > b->max_d) b->max_d = D[i];
    }
    b->row_last_all = (int *)(a + pos);
    b->row_last_count = rl;
    size_t rlpos = 0;
    for (int i = 0; i < n; i++) {
        b->views[i].row_last = b->row_last_all + rlpos;
        rlpos += H[i];
    }
    pos += align256(rl * 4);
    b->table = a + pos;
}

void link_pair(ViewBatch *b, int left, int right) {
    ViewDesc &l = b->views[left], &r = b->views[right];
    l.prep = 1;
    l.partner = right;
    r.prep = 0;
    r.rref = l.rtar;
    r.rtar = l.rref;
    r.aref = l.atar;
    r.atar = l.aref;
    r.mref = l.mtar;
    r.mtar = l.mref;
}

rts_status plan_views(rts_ctx *c, int slot, const int *W, const int *H, const int *D, int n, int half,
                      const CrossTune &tune, ViewBatch *b) {
    (void)tune;
    void *arena;
    RTS_TRY(scratch(c, slot, views_bytes(W, H, D, n, half), &arena));
    plan_views_at(arena, W, H, D, n, half, b);
    return RTS_OK;
}

rts_status upload_views(rts_ctx *c, const ViewBatch &bc, const CrossTune &tune, void *stage, ViewTable *t) {
    ViewBatch &b = const_cast<ViewBatch &>(bc);
    const int n = (int)b.views.size();
    // stage offsets from the per-view item counts
    for (int s = 0; s < ST_COUNT; s++) {
        int *o = &b.off[(size_t)s * (n + 1)];
        o[0] = 0;
        for (int i = 0; i < n; i++) {
            const ViewDesc &v = b.views[i];
            int items = stage_items(s, v, tune.vert_rows);
            if (s == ST_CC && (v.partner < 0 || !v.mask)) items = 0;
            o[i + 1] = o[i] + items;
        }
        b.total[s] = o[n];
    }
    const size_t vbytes = sizeof(ViewDesc) * n, obytes = sizeof(int) * b.off.size();
    unsigned char *d = (unsigned char *)b.table;
    int *doff = (int *)(d + ((vbytes + 255) & ~size_t(255)));
    if (stage) {
        // through pinned staging: the copies may then run asynchronously (and be replayed)
        memcpy(stage, b.views.data(), vbytes);
        memcpy((unsigned char *)stage + ((vbytes + 255) & ~size_t(255)), b.off.data(), obytes);
        RTS_CU(c, cudaMemcpyAsync(d, stage, ((vbytes + 255) & ~size_t(255)) + obytes, cudaMemcpyHostToDevice,
                                  c->stream));
    } else {
        RTS_CU(c, cudaMemcpyAsync(d, b.views.data(), vbytes, cudaMemcpyHostToDevice, c->stream));
        RTS_CU(c, cudaMemcpyAsync(doff, b.off.data(), obytes, cudaMemcpyHostToDevice, c->stream));
    }
    t->views = (const ViewDesc *)d;
    t->off = doff;
    t->nviews = n;
    for (int s = 0; s < ST_COUNT; s++) t->total[s] = b.total[s];
    return RTS_OK;
}

}  // namespace rts
