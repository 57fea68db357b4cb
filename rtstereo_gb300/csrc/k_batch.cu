// k_batch.cu -- the cross-based pipeline over a table of views, one launch per
// stage for a whole batch (one pair = its left and right view).
//
// Stages (each a persistent kernel looping over the work items of all views):
//   prep   block per (view, image, row): 16-byte pixel records of the view's
//          reference and target image (census code, packed RGB, packed arms),
//          read through mirrored addressing for right views
//   hseg   warp per (view, row, 32 disparities): cost, running sum along x
//          (seq/CrossBasedAggregation.cpp:117-125), row segments (:151-160) and
//          the geometry word of every entry
//   vert   block per (view, column, 64-row strip): vertical sums of the row
//          segments over the cross (:140-167), the division, and the first strict
//          arg-min over d (seq/WTA.cpp:15-22)
//   fill   warp per (view, row): the winner carry of seq/WTA.cpp:12
//   cc     block per (pair, row): seq/CrossCheck.cpp:10-23
// The per-entry arithmetic is the reference's (see k_pipe.cu), so a pair's
// result does not depend on what else is in the batch.
#include "rts_fused.cuh"
#include "rts_views.h"

namespace rts {

__device__ __forceinline__ int find_view(const int *__restrict__ off, int n, int item) {
    int lo = 0, hi = n - 1;  // largest v with off[v] <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// prep: block per (view, image, row, 128-column segment).  The block stages in
// shared memory, in view coordinates (mirrored for right views): the census
// rows y-hr .. y+hr for columns x0-wr .. x0+127+wr (wrapped, as the census
// wraps, seq/CensusTransform.cpp:20-26), the packed colours of row y for
// columns x0-L .. x0+127+L and of rows y-L .. y+L for columns x0 .. x0+127
// (arms stop at the image edge, so those are not wrapped).
constexpr int kPrepSeg = 128;
constexpr uint32_t kNoPixel = 0xff000000u;

__global__ void __launch_bounds__(kPrepSeg) k_prep_views(ViewTable t, int hr, int wr, int L, int tau, int want_code) {
    extern __shared__ __align__(16) unsigned char psm[];
    const int nv = t.nviews;
    const int *off = t.off + ST_PREP * (nv + 1);
    const int cw = kPrepSeg + 2 * wr;           // census tile width
    const int hw = kPrepSeg + 2 * L;            // horizontal colour row
    uint8_t *ct = psm;                          // [(2hr+1)][cw]
    uint32_t *hrow = reinterpret_cast<uint32_t *>(psm + (((2 * hr + 1) * cw + 15) & ~15));  // [hw]
    uint32_t *vcol = hrow + hw;                 // [(2L+1)][kPrepSeg]
    const int tx = threadIdx.x;
    for (int item = blockIdx.x; item < t.total[ST_PREP]; item += gridDim.x) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W, H = V.H, mir = V.mirror;
        const int nseg = (W + kPrepSeg - 1) / kPrepSeg;
        const int local = item - __ldg(off + v);
        const int img = local >= H * nseg ? 1 : 0;
        const int rest = local - img * H * nseg;
        const int y = rest / nseg, x0 = (rest - y * nseg) * kPrepSeg;
        const uint8_t *gray = img ? V.gtar : V.gref;
        const uint8_t *rgb = img ? V.ctar : V.cref;
        uint4 *out = img ? V.rtar : V.rref;
        auto sx = [&](int xm) { return mir ? W - 1 - xm : xm; };
        // colour of a pixel in view coordinates; without an RGB image the gray value
        // in all three channels (what the reference driver reads from a gray file,
        // seq/Main.cpp:87-90)
        auto colour = [&](int qy, int qx) -> uint32_t {
            if (qx < 0 || qx >= W || qy < 0 || qy >= H) return kNoPixel;
            const size_t q = (size_t)qy * W + sx(qx);
            if (!rgb) return (uint32_t)gray[q] * 0x010101u;
            const uint8_t *px = rgb + 3 * q;
            return (uint32_t)px[0] | ((uint32_t)px[1] << 8) | ((uint32_t)px[2] << 16);
        };
        __syncthreads();  // previous item done with the tiles
        if (want_code)
            for (int q = tx; q < (2 * hr + 1) * cw; q += kPrepSeg) {
                const int r = q / cw, cx = q - r * cw;
                const int yy = wrap1(y - hr + r, H);
                const int xx = x0 - wr + cx;
                // columns past the end of the last segment are never read by real pixels
                const int xw = imin(imax(wrap1(xx, W), 0), W - 1);
                ct[q] = gray[(size_t)yy * W + sx(xw)];
            }
        for (int q = tx; q < hw; q += kPrepSeg) hrow[q] = colour(y, x0 - L + q);
        for (int q = tx; q < (2 * L + 1) * kPrepSeg; q += kPrepSeg) {
            const int r = q / kPrepSeg, cx = q - r * kPrepSeg;
            vcol[q] = colour(y - L + r, x0 + cx);
        }
        __syncthreads();
        const int x = x0 + tx;
        if (x < W) {
            uint64_t code = 0;
            if (want_code) {
                const uint8_t c = ct[hr * cw + wr + tx];
                int k = 0;
                for (int r = 0; r <= 2 * hr; r++)
                    for (int dx = 0; dx <= 2 * wr; dx++, k++) code |= (uint64_t)(c > ct[r * cw + tx + dx]) << k;
            }
            const uint32_t packed = hrow[L + tx];
            // cross arms, seq/CrossBasedAggregation.cpp:12-100: step while the max channel
            // difference to the centre stays below tau and the arm is shorter than L;
            // the first failing pixel is included; stop at the image edge
            auto delta = [&](uint32_t q) {
                const uint32_t ad = __vabsdiffu4(packed, q);
                return imax(imax((int)(ad & 0xff), (int)((ad >> 8) & 0xff)), (int)((ad >> 16) & 0xff));
            };
            int len[4];
            const int room[4] = {x, W - 1 - x, y, H - 1 - y};
#pragma unroll
            for (int a = 0; a < 4; a++) {
                int n = 0, dl = 0;
                while (dl < tau && n < L && n < room[a]) {
                    n++;
                    const uint32_t q = a == 0 ? hrow[L + tx - n] : a == 1 ? hrow[L + tx + n]
                                     : a == 2 ? vcol[(L - n) * kPrepSeg + tx] : vcol[(L + n) * kPrepSeg + tx];
                    dl = delta(q);
                }
                len[a] = n;
            }
            const uint32_t arms = (uint32_t)len[0] | ((uint32_t)len[1] << 8) | ((uint32_t)len[2] << 16) |
                                  ((uint32_t)len[3] << 24);
            out[(size_t)y * W + x] = make_uint4((uint32_t)code, (uint32_t)(code >> 32), packed, arms);
        }
    }
}

// ---------------------------------------------------------------------------
// hseg: lane = disparity; 16-column steps of cost + running sum into registers,
// then a 64-entry ring per lane in shared memory and the segments whose right
// end is known (arms <= 23).  Records are staged 32 columns at a time.
constexpr int kRingV = 64;
constexpr int kHsegW = 2;
constexpr int kStepV = 16;

// MODE: 0 precomputed volume, 1 truncated AD + census on the integer path (the
// configuration of the cross-based pipeline), 2 any AD/census combination
template <typename ST, int MODE>
__global__ void __launch_bounds__(kHsegW * 32) k_hseg_views(ViewTable t, CostCfg cfg, int L) {
    constexpr bool VOL = MODE == 0;
    __shared__ float pring[kHsegW][kRingV][32];
    __shared__ uint16_t lring[kHsegW][kRingV][32];
    __shared__ uint4 recA[kHsegW][32];
    __shared__ uint4 recB[kHsegW][64];
    __shared__ float volS[VOL ? kHsegW : 1][VOL ? 32 : 1][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nv = t.nviews;
    const int *off = t.off + ST_HSEG * (nv + 1);
    float (*P)[32] = pring[warp];
    uint16_t (*LR)[32] = lring[warp];
    uint4 *RA = recA[warp], *RB = recB[warp];
    for (int item = blockIdx.x * kHsegW + warp; item < t.total[ST_HSEG]; item += gridDim.x * kHsegW) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W, D = V.D;
        const int nch = (D + 31) >> 5;
        const int local = item - __ldg(off + v);
        const int y = local / nch, dbase = (local - y * nch) * 32;
        const int d = dbase + lane;
        const bool active = d < D;
        const int dd = active ? d : D - 1;
        const int lo = dd - dbase;
        const size_t row = (size_t)y * W;
        const uint4 *rr = V.rref, *rt = V.rtar;
        ST *seg = reinterpret_cast<ST *>(V.seg);
        uint16_t *geo = V.geo;
        const float *vol = V.vol;

        auto emit = [&](int xs) {
            const uint16_t lr = LR[xs & (kRingV - 1)][lane];
            const int l = lr & 0xff, r = lr >> 8;
            int xl = xs - l - 1;
            if (xl < 0) xl = 0;  // seq/CrossBasedAggregation.cpp:153-154
            const int xr = xs + r;
            const float s = __fsub_rn(P[xr & (kRingV - 1)][lane], P[xl & (kRingV - 1)][lane]);
            if (active) seg[(row + xs) * D + d] = to_store<ST>(s);
        };
        auto wrapx = [&](int tt) {
            tt %= W;
            return tt < 0 ? tt + W : tt;
        };
        uint4 na, nb0, nb1;
        auto fetch = [&](int x0) {
            const int t0 = x0 - dbase - 31;
            na = rr[row + imin(x0 + lane, W - 1)];
            nb0 = rt[row + wrapx(t0 + lane)];
            nb1 = rt[row + wrapx(t0 + 32 + lane)];
        };
        fetch(0);
        float acc = 0.f;
        for (int x0 = 0; x0 < W; x0 += 32) {
            __syncwarp();
            RA[lane] = na;
            RB[lane] = nb0;
            RB[lane + 32] = nb1;
            if constexpr (VOL) {
#pragma unroll 8
                for (int u = 0; u < 32; u++)
                    if (x0 + u < W) volS[warp][u][lane] = vol[(row + x0 + u) * D + dd];
            }
            __syncwarp();
            if (x0 + 32 < W) fetch(x0 + 32);
#pragma unroll 1
            for (int h = 0; h < 32; h += kStepV) {
                const int xb = x0 + h;
                if (xb >= W) break;
                const int n = imin(kStepV, W - xb);
                float pv[kStepV];
                uint16_t lv[kStepV];
#pragma unroll
                for (int u = 0; u < kStepV; u++) {
                    if (u < n) {
                        const uint4 a = RA[h + u];
                        const uint4 b = RB[h + u + 31 - lo];  // target column x - dd
                        float c;
                        if constexpr (MODE == 0) {
                            c = volS[warp][h + u][lane];
                        } else if constexpr (MODE == 1) {
                            // CombineCost of min(SAD, trunc) and the Hamming distance through
                            // the host expf tables (seq/CombineCost.cpp:21-23)
                            const int sad = imin((int)__vsadu4(a.z, b.z), cfg.itrunc);
                            const int ham = __popc(a.x ^ b.x) + __popc(a.y ^ b.y);
                            c = __fadd_rn(__ldg(cfg.lut1 + sad), __ldg(cfg.lut2 + ham));
                        } else {
                            c = pair_cost(a, b, cfg);
                        }
                        acc = (xb + u == 0) ? c : __fadd_rn(c, acc);  // seq/CrossBasedAggregation.cpp:123
                        pv[u] = acc;
                        const uint32_t m = __vminu4(a.w, b.w);  // byte-wise min of the four arms
                        lv[u] = (uint16_t)(m & 0xffff);
                        if (active)
                            geo[(row + xb + u) * D + d] = (uint16_t)(((m & 0xff) + ((m >> 8) & 0xff) + 1) |
                                                                     (((m >> 16) & 0xff) << 6) | ((m >> 24) << 11));
                    }
                }
#pragma unroll
                for (int u = 0; u < kStepV; u++) {
                    if (u < n) {
                        P[(xb + u) & (kRingV - 1)][lane] = pv[u];
                        LR[(xb + u) & (kRingV - 1)][lane] = lv[u];
                    }
                }
                // segments whose right end xs + L is now in the ring
#pragma unroll
                for (int u = 0; u < kStepV; u++) {
                    const int xs = xb - L + u;
                    if (u < n && xs >= 0) emit(xs);
                }
            }
        }
        for (int xs = imax(0, W - L); xs < W; xs++) emit(xs);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// vert: block per (view, column, strip of R output rows).  The strip's rows
// y0-L .. y0+R+L-1 (segments and geometry words of all disparities) are copied
// into shared memory with cp.async (all in flight at once); a column-wise
// running count of the row pixel counts (integers, so exact) replaces the
// per-row count additions; each warp then owns whole output rows.
constexpr int kVertT = 256;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename ST, int NCH>
__global__ void __launch_bounds__(kVertT) k_vert_views(ViewTable t, int L, int R) {
    // NCH: 32-disparity chunks per column (D <= 32 * NCH)
    extern __shared__ __align__(16) unsigned char vsm[];
    __shared__ uint32_t armr[256];  // packed arms of the reference pixel (row, x) of the strip
    const int nv = t.nviews;
    const int *off = t.off + ST_VERT * (nv + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int item = blockIdx.x; item < t.total[ST_VERT]; item += gridDim.x) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W, H = V.H, D = V.D;
        const int strips = (H + R - 1) / R;
        const int local = item - __ldg(off + v);
        const int x = local / strips, strip = local - x * strips;
        const int y0 = strip * R, y1 = imin(H, y0 + R);
        const int ya0 = imax(0, y0 - L), ya1 = imin(H, y1 + L);
        const int nr = ya1 - ya0;
        const ST *seg = reinterpret_cast<const ST *>(V.seg);
        ST *S = reinterpret_cast<ST *>(vsm);
        uint16_t *G = reinterpret_cast<uint16_t *>(vsm + (size_t)(R + 2 * L) * D * sizeof(ST));
        // column prefix of the row pixel counts: CP[r*D + d] = sum of counts of rows < r
        // (at most (R + 2L) * (2L + 1) < 65536)
        uint16_t *CP = reinterpret_cast<uint16_t *>(vsm + (size_t)(R + 2 * L) * D * (sizeof(ST) + 2));
        __syncthreads();  // previous item done with the tile
        {
            constexpr int SV = 16 / sizeof(ST);
            const int sv_row = D / SV, g_row = D / 8;
            const int per_row = sv_row + g_row;
            for (int q = threadIdx.x; q < nr * per_row; q += kVertT) {
                const int ri = q / per_row, k = q - ri * per_row;
                const size_t src = ((size_t)(ya0 + ri) * W + x) * D;
                if (k < sv_row) cp_async16(reinterpret_cast<uint4 *>(S + (size_t)ri * D) + k,
                                           reinterpret_cast<const uint4 *>(seg + src) + k);
                else cp_async16(reinterpret_cast<uint4 *>(G + (size_t)ri * D) + (k - sv_row),
                                reinterpret_cast<const uint4 *>(V.geo + src) + (k - sv_row));
            }
            for (int ri = threadIdx.x; ri < nr; ri += kVertT) armr[ri] = V.rref[(size_t)(ya0 + ri) * W + x].w;
            cp_async_wait_all();
        }
        __syncthreads();
        for (int d = threadIdx.x; d < D; d += kVertT) {
            int acc = 0;
            for (int ri = 0; ri < nr; ri++) {
                CP[ri * D + d] = (uint16_t)acc;
                acc += G[ri * D + d] & 63;
            }
            CP[nr * D + d] = (uint16_t)acc;
        }
        __syncthreads();
        for (int yo = y0 + warp; yo < y1; yo += kVertT / 32) {
            const int ro = yo - ya0;
            // every disparity's vertical arm is inside the reference pixel's own arm
            const uint32_t ar = armr[ro];
            const int rlo = ro - (int)((ar >> 16) & 0xff), rhi = ro + (int)(ar >> 24);
            const int nch = (D + 31) >> 5;  // this view's chunks (<= NCH)
            int lo[NCH];
            unsigned span[NCH];
            float sum[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                const int d = c * 32 + lane;
                const int g = (c < nch && d < D) ? G[ro * D + d] : 0;
                lo[c] = ro - ((g >> 6) & 31);
                // rows lo .. lo+span; lanes past D get an empty range
                span[c] = (c < nch && d < D) ? (unsigned)((g >> 11) + ((g >> 6) & 31)) : 0xffffffffu;
                sum[c] = 0.f;
            }
            // seq/CrossBasedAggregation.cpp:146-164: row segments of each (x, d) top to
            // bottom; a row outside that disparity's own arm is skipped, not added
            for (int r = rlo; r <= rhi; r++) {
#pragma unroll
                for (int c = 0; c < NCH; c++) {
                    if (c < nch && (unsigned)(r - lo[c]) <= span[c])
                        sum[c] = __fadd_rn(sum[c], to_f32(S[r * D + c * 32 + lane]));
                }
            }
            uint32_t best_key = 0xffffffffu;
            int best_d = 0;
#pragma unroll
            for (int c = 0; c < NCH; c++) {
                if (c >= nch) break;
                const int d = c * 32 + lane;
                uint32_t key = 0xffffffffu;
                if (d < D) {
                    const int cnt = CP[(lo[c] + (int)span[c] + 1) * D + d] - CP[lo[c] * D + d];
                    key = order_key(__fdiv_rn(sum[c], (float)cnt));  // :166
                }
                const uint32_t m = __reduce_min_sync(0xffffffffu, key);
                if (m < best_key) {  // strict: an earlier chunk keeps ties
                    const unsigned hit = __ballot_sync(0xffffffffu, key == m);
                    best_key = m;
                    best_d = c * 32 + __ffs(hit) - 1;
                }
            }
            if (lane == 0) {
                const bool found = best_d != 0;  // some d >= 1 strictly below cost[0]
                V.raw[(size_t)yo * W + x] = found ? (uint16_t)(0x100 | best_d) : (uint16_t)0;
                if (found) atomicMax(V.row_last + yo, x);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// fill: warp per (view, row); see k_wta.cu for the carry rule
__global__ void __launch_bounds__(256) k_fill_views(ViewTable t) {
    const int nv = t.nviews;
    const int *off = t.off + ST_FILL * (nv + 1);
    const int lane = threadIdx.x & 31;
    for (int item = blockIdx.x * 8 + (threadIdx.x >> 5); item < t.total[ST_FILL]; item += gridDim.x * 8) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W;
        const int y = item - __ldg(off + v);
        const uint16_t *raw = V.raw;
        int carry = 0;
        for (int base = y - 1; base >= 0; base -= 32) {
            const int yy = base - lane;
            const bool has = yy >= 0 && V.row_last[yy] >= 0;
            const unsigned m = __ballot_sync(0xffffffffu, has);
            if (m) {
                const int yy0 = base - (__ffs(m) - 1);
                carry = raw[(size_t)yy0 * W + V.row_last[yy0]] & 0xff;
                break;
            }
        }
        const uint16_t *r = raw + (size_t)y * W;
        uint8_t *o = V.disp + (size_t)y * W;
        for (int x0 = 0; x0 < W; x0 += 32) {
            const int x = x0 + lane;
            const uint16_t val = x < W ? r[x] : (uint16_t)0;
            const unsigned fm = __ballot_sync(0xffffffffu, (val & 0x100) != 0);
            const unsigned le = fm & (0xffffffffu >> (31 - lane));
            const int src = le ? 31 - __clz(le) : 0;
            const int got = __shfl_sync(0xffffffffu, val & 0xff, src);
            if (x < W) o[V.mirror ? W - 1 - x : x] = (uint8_t)(le ? got : carry);
            if (fm) carry = __shfl_sync(0xffffffffu, val & 0xff, 31 - __clz(fm));
        }
    }
}

// ---------------------------------------------------------------------------
// cc: block per (left view, row)
__global__ void __launch_bounds__(256) k_cc_views(ViewTable t) {
    const int nv = t.nviews;
    const int *off = t.off + ST_CC * (nv + 1);
    for (int item = blockIdx.x; item < t.total[ST_CC]; item += gridDim.x) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W;
        const int y = item - __ldg(off + v);
        const uint8_t *dl = V.disp + (size_t)y * W;
        const uint8_t *dr = t.views[V.partner].disp + (size_t)y * W;
        for (int x = threadIdx.x; x < W; x += blockDim.x) {
            const int val = dl[x];
            int xt = x - val;
            if (xt < 0) xt += W;
            V.mask[(size_t)y * W + x] = (dr[xt] == val) ? 1 : 0;
        }
    }
}

// ---------------------------------------------------------------------------
int stage_items(int stage, int W, int H, int D, int vert_rows) {
    switch (stage) {
    case ST_PREP: return 2 * H * ((W + kPrepSeg - 1) / kPrepSeg);
    case ST_HSEG: return H * ((D + 31) / 32);
    case ST_VERT: return W * ((H + vert_rows - 1) / vert_rows);
    case ST_FILL: return H;
    case ST_CC: return H;
    }
    return 0;
}

static int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 132;
    }
    return n;
}

rts_status launch_cross_views(rts_ctx *c, const rts_params &p, const ViewTable &t, int half, int has_vol, int max_d,
                              const CrossTune &tune, int *row_last_all, size_t row_last_count) {
    CostCfg cfg;
    cfg.k1 = p.cost1;
    cfg.k2 = p.cost2;
    cfg.trunc1 = (p.cost1 == RTS_COST_AD && p.aggr == RTS_AGGR_CROSS) ? 1 : 0;  // seq/Main.cpp:183-186
    cfg.trunc = p.ad_trunc;
    cfg.l1 = p.lambda1;
    cfg.l2 = p.lambda2;
    cfg.lut1 = cfg.lut2 = nullptr;
    // integer fast path: AD with an integral truncation (or none) and census take
    // integer values below the table size (AD <= 765, census <= 64)
    const bool trunc_ok = !cfg.trunc1 || (p.ad_trunc >= 0.f && p.ad_trunc < (float)kCombineLut &&
                                         p.ad_trunc == floorf(p.ad_trunc));
    cfg.int_path = trunc_ok ? 1 : 0;
    cfg.itrunc = cfg.trunc1 ? (int)p.ad_trunc : 0x7fffffff;
    if (p.cost2 != RTS_COST_NONE) RTS_TRY(combine_luts(c, p.lambda1, p.lambda2, &cfg.lut1, &cfg.lut2));
    cudaStream_t s = c->stream;
    const int sms = num_sms();
    auto grid = [&](int items, int per_block, int per_sm) {
        const long need = ((long)items + per_block - 1) / per_block;
        const long cap = (long)sms * per_sm;
        return (unsigned)(need < cap ? (need > 0 ? need : 1) : cap);
    };
    const int L = p.cross_arm, R = tune.vert_rows;
    RTS_CU(c, cudaMemsetAsync(row_last_all, 0xff, row_last_count * sizeof(int), s));
    const bool want_code = !has_vol && (p.cost1 == RTS_COST_CENSUS || p.cost2 == RTS_COST_CENSUS);
    {
        StageScope sc(c, "prep");
        const int hr = p.census_hrad, wr = p.census_wrad;
        const size_t smem = (((2 * hr + 1) * (kPrepSeg + 2 * wr) + 15) & ~15) + 4 * (kPrepSeg + 2 * L) +
                            4 * (size_t)(2 * L + 1) * kPrepSeg;
        cudaFuncSetAttribute(k_prep_views, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_prep_views<<<grid(t.total[ST_PREP], 1, 16), kPrepSeg, smem, s>>>(t, hr, wr, L, p.cross_tau,
                                                                          want_code ? 1 : 0);
        count_launch(c);
    }
    {
        StageScope sc(c, "cross_hseg");
        const unsigned g = grid(t.total[ST_HSEG], kHsegW, 8 * tune.grid_mult);
        const int mode = has_vol ? 0
                         : (cfg.int_path && cfg.k1 == RTS_COST_AD && cfg.trunc1 && cfg.k2 == RTS_COST_CENSUS) ? 1
                                                                                                               : 2;
        auto go = [&](auto kern) { kern<<<g, kHsegW * 32, 0, s>>>(t, cfg, L); };
        if (half) {
            if (mode == 0) go(k_hseg_views<__half, 0>);
            else if (mode == 1) go(k_hseg_views<__half, 1>);
            else go(k_hseg_views<__half, 2>);
        } else {
            if (mode == 0) go(k_hseg_views<float, 0>);
            else if (mode == 1) go(k_hseg_views<float, 1>);
            else go(k_hseg_views<float, 2>);
        }
        count_launch(c);
    }
    {
        StageScope sc(c, "cross_vert_wta");
        const size_t smem = (size_t)(R + 2 * L) * max_d * ((half ? 2 : 4) + 2) + (size_t)(R + 2 * L + 1) * max_d * 2;
        const unsigned g = grid(t.total[ST_VERT], 1, 2 * tune.grid_mult);
        auto go = [&](auto kern) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<g, kVertT, smem, s>>>(t, L, R);
        };
        const int nch = (max_d + 31) / 32;
        if (half) {
            if (nch <= 1) go(k_vert_views<__half, 1>);
            else if (nch <= 2) go(k_vert_views<__half, 2>);
            else if (nch <= 4) go(k_vert_views<__half, 4>);
            else go(k_vert_views<__half, 8>);
        } else {
            if (nch <= 1) go(k_vert_views<float, 1>);
            else if (nch <= 2) go(k_vert_views<float, 2>);
            else if (nch <= 4) go(k_vert_views<float, 4>);
            else go(k_vert_views<float, 8>);
        }
        count_launch(c);
    }
    {
        StageScope sc(c, "wta_fill");
        k_fill_views<<<grid(t.total[ST_FILL], 8, 8), 256, 0, s>>>(t);
        count_launch(c);
    }
    if (t.total[ST_CC] > 0) {
        StageScope sc(c, "cross_check");
        k_cc_views<<<grid(t.total[ST_CC], 1, 8), 256, 0, s>>>(t);
        count_launch(c);
    }
    return check_launch(c, "cross views");
}

}  // namespace rts
