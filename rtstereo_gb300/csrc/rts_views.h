// rts_views.h -- view tables for the cross-based pipeline (k_batch.cu).
//
// A view is one direction of one stereo pair: the left view matches the left
// image against the right one; the right view is the same computation on the
// horizontally mirrored images (right image as reference), which the kernels
// read through mirrored addressing instead of flipped copies.  The per-pixel
// records of an image are made once, in image coordinates, by the view that
// owns them (prep = 1) and shared with the pair's other view.  Every stage
// kernel runs over all views of a batch in one launch: work items of all views
// are numbered consecutively and a kernel finds an item's view by binary
// search in the per-view prefix offsets.
#pragma once

#include <stdint.h>

#include <vector>

#include "rts_internal.h"

namespace rts {

struct ViewDesc {
    const uint8_t *gref, *gtar;  // source gray images [H][W] (unmirrored)
    const uint8_t *cref, *ctar;  // source RGB images [H][W][3]
    const uint8_t *mref, *mtar;  // median-filtered arm images (channels as cref, else as gref), or nullptr
    const float *vol;            // optional precomputed cost volume of the view [H][W][D] (or nullptr)
    int mirror;                  // 1: the view reads its sources mirrored in x
    int W, H, D;
    uint4 *rref, *rtar;          // per-pixel records {census lo, census hi, colour, l | r<<16}, image coordinates
    uint2 *aref, *atar;          // per-pixel arm words {l | r<<16, t | b<<16}, image coordinates
    void *seg;                   // row segments [H][W][D] in view coordinates, float or __half
    uint16_t *raw;               // winner | found << 8 per pixel
    int *row_last;               // per row: last x with a winner of its own, -1 if none
    uint8_t *disp;               // output disparity (written mirrored back when mirror)
    uint8_t *mask;               // cross-check mask of the pair (left views only), or nullptr
    int partner;                 // index of the right view of the same pair, or -1
    int prep;                    // 1: this view makes the records of both its images
};

// stage offsets: item k of stage s belongs to view v with off[s][v] <= k < off[s][v+1]
enum { ST_PREP = 0, ST_HSEG, ST_VERT, ST_FILL, ST_CC, ST_COUNT };

struct ViewTable {
    const ViewDesc *views;  // device
    const int *off;         // device, [ST_COUNT][nviews + 1]
    int nviews;
    int total[ST_COUNT];
};

struct CrossTune {
    int vert_rows = 4096;   // output rows per vertical-aggregation item (a strip of one column)
    int grid_mult = 8;      // persistent blocks per SM of the row-segment kernel
    int persistent = 0;     // 0: one block per work item (the hardware balances the
                            // blocks); 1: resident blocks striding over the items
};

// Per-view item counts (host): the layout the kernels and the planner share.
int stage_items(int stage, const ViewDesc &v, int vert_rows);

// The costs the cross-based view kernels make from per-pixel records: AD and
// census (alone or combined), and rank differences combined with census.
bool cross_record_costs(const rts_params &p);

// Host tables the cross-based kernels read (combined cost table, reciprocals);
// made before a graph capture so that the launches find them cached.
rts_status cross_tables(rts_ctx *c, const rts_params &p);

// Row-segment storage of a cross-based launch whose widest view is max_w:
// 2 exact u16 integers (integer costs, either form), 1 f16 (FP16 form), 0 f32.
// Layouts (views_bytes, plan_views_at) take `kind != 0` as their 2-byte flag.
int cross_seg_kind(const rts_params &p, int max_w);

// Launches all stages of the cross-based pipeline over a view table that is
// already on the device; segk is the segment kind (cross_seg_kind, or 0/1 by
// the form for precomputed volumes), gray that no view has an RGB image.
rts_status launch_cross_views(rts_ctx *c, const rts_params &p, const ViewTable &t, int segk, int has_vol, int gray,
                              int max_d, const CrossTune &tune, int *row_last_all, size_t row_last_count);

// One batch of views on the device, planned on the host.
struct ViewBatch {
    std::vector<ViewDesc> views;     // host copy
    std::vector<int> off;            // [ST_COUNT][n + 1]
    int total[ST_COUNT] = {0, 0, 0, 0, 0};
    int max_d = 0;
    int *row_last_all = nullptr;     // device, contiguous over views
    size_t row_last_count = 0;
    void *table = nullptr;           // device space for the view table and offsets
};

// Sizes the scratch of `n` views (W, H, D per view), carves it from the arena
// slot, fills the device-side buffers of every ViewDesc (records, arm words,
// segments, winners, row summaries) and the stage offsets.  Image, output and
// volume pointers are left for the caller to fill before upload.
rts_status plan_views(rts_ctx *c, int slot, const int *W, const int *H, const int *D, int n, int half,
                      const CrossTune &tune, ViewBatch *b);
// Device bytes of the scratch, view table and offsets of n views.
size_t views_bytes(const int *W, const int *H, const int *D, int n, int half);
// Carves n views out of an arena of views_bytes() bytes.
void plan_views_at(void *arena, const int *W, const int *H, const int *D, int n, int half, ViewBatch *b);
// Makes views `left` and `right` one pair: the left view makes the records of
// both images, the right view reads them (its reference is the right image).
void link_pair(ViewBatch *b, int left, int right);
// Computes the stage offsets, copies the view table and offsets to the device
// (through the pinned buffer `stage` when given, else directly) and fills `t`.
rts_status upload_views(rts_ctx *c, const ViewBatch &b, const CrossTune &tune, void *stage, ViewTable *t);

// The batched cross-based pipeline over n validated pairs (DEVICE buffers, fast
// costs): autotuned tiles and one captured CUDA graph per batch shape.
rts_status batch_views_run(rts_ctx *c, int n, const rts_pair *pairs, const rts_params *params, rts_out *outs);

}  // namespace rts
