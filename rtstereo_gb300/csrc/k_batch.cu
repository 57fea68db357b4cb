// k_batch.cu -- the cross-based pipeline over a table of views, one launch per
// stage for a whole batch (one pair = its left and right view).
//
// Stages (each kernel loops over the work items of all views: one block per
// item by default, or resident blocks striding over them):
//   prep   block per (image, 64x16 tile): per-pixel records of every image
//          (census code, colour, horizontal arms) and arm words (horizontal and
//          vertical arms), in image coordinates, made once per image and read by
//          both views of the pair
//   hseg   warp per (view, row, 32 disparities): cost, running sum along x
//          (seq/CrossBasedAggregation.cpp:117-125) and the row segment of every
//          entry (:151-160)
//   vert   block per (view, column, strip of rows): row segments streamed down
//          the column through a shared ring, vertical sums over the cross
//          (:140-167), the division and the first strict arg-min over d
//          (seq/WTA.cpp:15-22)
//   fill   warp per (view, row): the winner carry of seq/WTA.cpp:12
//   cc     block per (pair, row): seq/CrossCheck.cpp:10-23
//
// A right view is the left-to-right pipeline on the mirrored images.  It reads
// the pair's records through mirrored column addressing with the left and right
// arms swapped; its census codes are the unmirrored ones, which differ from the
// codes of the mirrored image only by one fixed permutation of the bits (the
// window, and its wrap at the borders, are mirror symmetric), so every Hamming
// distance is the same.  The per-entry arithmetic is the reference's, so a
// pair's result does not depend on what else is in the batch.
#include <algorithm>
#include <type_traits>

#include "rts_fused.cuh"
#include "rts_pipe.h"
#include "rts_vert_ring.h"
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
// prep: block per (view, image, 64x16 tile).  The colours of the tile and of
// L pixels around it (no wrap: arms stop at the image edge) and the gray census
// window around it (wrapped, seq/CensusTransform.cpp:20-26) are staged in
// shared memory; each thread then makes four pixels.
constexpr int kPrepTW = 64, kPrepTH = 16, kPrepT = 256;
constexpr uint32_t kNoPixel = 0xff000000u;

static size_t prep_smem(int gr, int gc, int L) {
    return (size_t)4 * (kPrepTW + 2 * L) * (kPrepTH + 2 * L) + (size_t)(kPrepTH + 2 * gr) * (kPrepTW + 2 * gc);
}

// the colour word of pixel p: RGB bytes, or the gray byte (replicated unless
// the records hold gray alone)
template <int GRAYREC>
__device__ __forceinline__ uint32_t pixel_word(const uint8_t *img, bool rgb, size_t p) {
    if (!rgb) return GRAYREC ? (uint32_t)img[p] : (uint32_t)img[p] * 0x010101u;
    const uint8_t *px = img + 3 * p;
    return (uint32_t)px[0] | ((uint32_t)px[1] << 8) | ((uint32_t)px[2] << 16);
}

// GRAYREC: the record colour is the gray byte (all views of the launch are
// gray; the cost kernel then takes 3|dI| as the colour AD), else packed RGB with
// gray replicated into the three channels (seq/Main.cpp:87-90).  rank >= 0: the
// record's colour word holds the rank of the pixel instead (radius rank,
// seq/RankFilter.cpp:11-35), which a mirrored view reads unchanged (the window
// and its wrap are mirror symmetric).  The gray tile has a wrapped border of
// gr rows and gc columns (the larger of the census and rank windows).  With
// median-filtered arm images (mref / mtar) the colour tile, and so the arms,
// come from those, and the records from the unfiltered sources.
template <int GRAYREC>
__global__ void __launch_bounds__(kPrepT) k_prep_views(ViewTable t, int hr, int wr, int L, int tau, int want_code,
                                                       int rank, int gr, int gc) {
    extern __shared__ __align__(16) unsigned char psm[];
    const int nv = t.nviews;
    const int *off = t.off + ST_PREP * (nv + 1);
    const int cw = kPrepTW + 2 * L, chh = kPrepTH + 2 * L;
    const int gw = kPrepTW + 2 * gc, gh = kPrepTH + 2 * gr;
    uint32_t *ct = reinterpret_cast<uint32_t *>(psm);  // [chh][cw] colours
    uint8_t *gt = psm + (size_t)4 * cw * chh;          // [gh][gw] gray, wrapped
    for (int item = blockIdx.x; item < t.total[ST_PREP]; item += gridDim.x) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W, H = V.H;
        const int ntx = (W + kPrepTW - 1) / kPrepTW, nty = (H + kPrepTH - 1) / kPrepTH;
        const int local = item - __ldg(off + v);
        const int img = local >= ntx * nty ? 1 : 0;
        const int tl = local - img * ntx * nty;
        const int by = tl / ntx;
        const int x0 = (tl - by * ntx) * kPrepTW, y0 = by * kPrepTH;
        const uint8_t *gray = img ? V.gtar : V.gref;
        const uint8_t *rgb = img ? V.ctar : V.cref;
        // the arms may come from median-filtered copies; the records keep the source colour
        const uint8_t *med = img ? V.mtar : V.mref;
        uint4 *rec = img ? V.rtar : V.rref;
        uint2 *arm = img ? V.atar : V.aref;
        __syncthreads();  // previous item done with the tiles
        for (int q = threadIdx.x; q < cw * chh; q += kPrepT) {
            const int r = q / cw, cx = q - r * cw;
            const int yy = y0 - L + r, xx = x0 - L + cx;
            uint32_t col = kNoPixel;
            if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
                col = pixel_word<GRAYREC>(med ? med : (rgb ? rgb : gray), rgb != nullptr, (size_t)yy * W + xx);
            }
            ct[q] = col;
        }
        if (want_code || rank >= 0)
            for (int q = threadIdx.x; q < gw * gh; q += kPrepT) {
                const int r = q / gw, cx = q - r * gw;
                // rows / columns past the last pixel's window are never read; clamp them
                // into the single-wrap range (the window radii are below H and W)
                const int yy = wrap1(imin(y0 - gr + r, H - 1 + gr), H);
                const int xx = wrap1(imin(x0 - gc + cx, W - 1 + gc), W);
                gt[q] = gray[(size_t)yy * W + xx];
            }
        __syncthreads();
        const int px = threadIdx.x & (kPrepTW - 1);
        for (int py = threadIdx.x / kPrepTW; py < kPrepTH; py += kPrepT / kPrepTW) {
            const int x = x0 + px, y = y0 + py;
            if (x >= W || y >= H) continue;
            uint32_t lo = 0, hi = 0;
            if (want_code) {
                // seq/CensusTransform.cpp:11-37: bit (dy+hr)*(2wr+1)+(dx+wr), strict centre > neighbour
                const uint8_t *g0 = gt + (py + gr - hr) * gw + px + gc - wr;
                const uint32_t c = g0[hr * gw + wr];
                int k = 0;
                for (int r = 0; r <= 2 * hr; r++)
                    for (int dx = 0; dx <= 2 * wr; dx++, k++) {
                        const uint32_t bit = c > (uint32_t)g0[r * gw + dx] ? 1u : 0u;
                        if (k < 32) lo |= bit << k;
                        else hi |= bit << (k - 32);
                    }
            }
            // cross arms, seq/CrossBasedAggregation.cpp:12-100: step while the max channel
            // difference to the centre stays below tau and the arm is shorter than L; the
            // first failing pixel is included; stop at the image edge
            const uint32_t *cc = ct + (py + L) * cw + (px + L);
            const uint32_t centre = *cc;
            auto delta = [&](uint32_t q) -> int {
                if (GRAYREC) return abs((int)q - (int)centre);
                const uint32_t ad = __vabsdiffu4(centre, q);
                return imax(imax((int)(ad & 0xff), (int)((ad >> 8) & 0xff)), (int)((ad >> 16) & 0xff));
            };
            const int room[4] = {x, W - 1 - x, y, H - 1 - y};
            const int stride[4] = {-1, 1, -cw, cw};
            int len[4];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                int n = 0, dl = 0;
                while (dl < tau && n < L && n < room[a]) {
                    n++;
                    dl = delta(cc[stride[a] * n]);
                }
                len[a] = n;
            }
            const uint32_t lr = (uint32_t)len[0] | ((uint32_t)len[1] << 16);
            const uint32_t tb = (uint32_t)len[2] | ((uint32_t)len[3] << 16);
            const size_t p = (size_t)y * W + x;
            uint32_t cword = med ? pixel_word<GRAYREC>(rgb ? rgb : gray, rgb != nullptr, p) : centre;
            if (rank >= 0) {
                // seq/RankFilter.cpp:16-29: 1 + neighbours strictly below the centre, as u8
                const uint8_t *g0 = gt + (py + gr - rank) * gw + px + gc - rank;
                const uint32_t c = g0[rank * gw + rank];
                int cnt = 1;
                for (int r = 0; r <= 2 * rank; r++)
                    for (int dx = 0; dx <= 2 * rank; dx++) cnt += (uint32_t)g0[r * gw + dx] < c ? 1 : 0;
                cword = (uint32_t)(uint8_t)cnt;
            }
            rec[p] = make_uint4(lo, hi, cword, lr);
            arm[p] = make_uint2(lr, tb);
        }
    }
}

// ---------------------------------------------------------------------------
// hseg: lane = disparity.  The running sum P of every column goes into a
// 64-column ring per lane; the segment of column xs is written 24 columns
// later (arms <= 23, so both of its ends are in the ring then):
//   seg(xs) = P[xs + r] - P[max(xs - l - 1, 0)]
// with (l, r) the byte-wise minimum of the reference and target arms kept in a
// 32-column ring as the pre-shifted word (l + 1) << 7 | r << 23.  Records are
// staged 32 columns at a time and worked in groups of kHSub columns: the costs
// (independent), the running sum, the segments of the columns 24 back, then
// the arm words.  Columns past the row end are computed from clamped records
// and never written.
constexpr int kHsegW = 2;   // warps per block
constexpr int kHLag = 24;   // columns between a column's prefix and its segment
constexpr int kHSub = 8;    // columns per group

// MODE: 0 precomputed volume, 1 truncated AD + census through the combined host
// table (the configuration of the cross-based pipeline), 2 any AD/census pair,
// 3 census alone, 4 truncated AD alone (integer costs, u16 segments)
template <typename ST, int MODE, int GRAYREC>
__global__ void __launch_bounds__(kHsegW * 32, 8) k_hseg_views(ViewTable t, CostCfg cfg) {
    __shared__ __align__(16) float pring[kHsegW][64][32];
    __shared__ uint32_t lring[kHsegW][32][32];
    __shared__ uint4 recA[kHsegW][32];
    __shared__ uint4 recB[kHsegW][64];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nv = t.nviews;
    const int *off = t.off + ST_HSEG * (nv + 1);
    float *PR = &pring[warp][0][lane];  // slot s at PR[32 s]
    uint32_t *LR = &lring[warp][0][lane];
    uint4 *RA = recA[warp], *RB = recB[warp];
    for (int item = blockIdx.x * kHsegW + warp; item < t.total[ST_HSEG]; item += gridDim.x * kHsegW) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int W = V.W, D = V.D, mir = V.mirror;
        const int nch = (D + 31) >> 5;
        const int local = item - __ldg(off + v);
        const int y = local / nch, dbase = (local - y * nch) * 32;
        const int d = dbase + lane;
        const bool active = d < D;
        const int dd = active ? d : D - 1;
        const size_t row = (size_t)y * W;
        const uint4 *rr = V.rref + row, *rt = V.rtar + row;
        ST *seg = reinterpret_cast<ST *>(V.seg) + row * D + d;
        const float *vol = MODE == 0 ? V.vol + row * D + dd : nullptr;
        // image column of view column xv (any integer: columns past the row end wrap)
        auto col = [&](int xv) {
            xv %= W;
            if (xv < 0) xv += W;
            return mir ? W - 1 - xv : xv;
        };
        // a mirrored view swaps the left and right arms
        auto fix = [&](uint4 r) {
            if (mir) r.w = __byte_perm(r.w, 0, 0x1032);
            return r;
        };
        uint4 na, nb0, nb1;
        auto fetch = [&](int x0) {
            const int t0 = x0 - dbase - 31;  // target column of RB[0]: x - d for x = x0, lane 31
            na = rr[col(imin(x0 + lane, W - 1))];
            nb0 = rt[col(t0 + lane)];
            nb1 = rt[col(t0 + 32 + lane)];
        };
        fetch(0);
        float acc = 0.f;
        const int xend = W + kHLag;
        for (int x0 = 0; x0 < xend; x0 += 32) {
            __syncwarp();
            RA[lane] = fix(na);
            RB[lane] = fix(nb0);
            RB[lane + 32] = fix(nb1);
            __syncwarp();
            if (x0 + 32 < xend) fetch(x0 + 32);
            // group h: columns x0 + kHSub h .. x0 + kHSub (h + 1) - 1
            auto group = [&](auto hc, auto edge) {
                constexpr int h = decltype(hc)::value;
                const int hx = x0 + kHSub * h;
                float cv[kHSub];
                uint32_t lv[kHSub];
#pragma unroll
                for (int u = 0; u < kHSub; u++) {
                    const uint4 a = RA[kHSub * h + u];
                    const uint4 b = RB[kHSub * h + u + 31 - lane];  // target column x - d
                    if constexpr (MODE == 0) {
                        cv[u] = vol[(size_t)imin(hx + u, W - 1) * D];
                    } else if constexpr (MODE == 1) {
                        // CombineCost of min(SAD, trunc) and the Hamming distance: the float add of
                        // the two host-made terms T1[s] + T2[h] (seq/CombineCost.cpp:21-23), two
                        // small tables a warp's lanes read in a few L1 lines
                        // the first cost: colour AD (truncated), or the AD of the ranks
                        // (seq/PixelBasedCost.cpp:13-24 on rank images)
                        int s = GRAYREC == 2 ? abs((int)a.z - (int)b.z)
                                : GRAYREC ? abs((int)a.z - (int)b.z) * 3 : (int)__vsadu4(a.z, b.z);
                        s = imin(s, cfg.itrunc);
                        const int hd = __popc(a.x ^ b.x) + __popc(a.y ^ b.y);
                        cv[u] = __fadd_rn(__ldg(cfg.lut1 + s), __ldg(cfg.lut2 + hd));
                    } else if constexpr (MODE == 3) {
                        // census alone: the Hamming distance (seq/CensusTransform.cpp:39-62)
                        cv[u] = (float)(__popc(a.x ^ b.x) + __popc(a.y ^ b.y));
                    } else if constexpr (MODE == 4) {
                        // truncated AD alone (seq/PixelBasedCost.cpp:13-24, seq/Main.cpp:183-186)
                        cv[u] = (float)imin((int)__vsadu4(a.z, b.z), cfg.itrunc);
                    } else {
                        cv[u] = pair_cost(a, b, cfg);
                    }
                    lv[u] = __vminu2(a.w, b.w) * 128u + 128u;
                }
                // running sum, seq/CrossBasedAggregation.cpp:123 (0 + c is c for every cost but -0)
                float *PRh = PR + ((x0 & 32) + kHSub * h) * 32;
#pragma unroll
                for (int u = 0; u < kHSub; u++) {
                    if constexpr (MODE == 0) acc = (hx + u == 0) ? cv[u] : __fadd_rn(acc, cv[u]);
                    else acc = __fadd_rn(acc, cv[u]);
                    PRh[u * 32] = acc;
                }
                // segments of columns xs = x - 24 (seq/CrossBasedAggregation.cpp:151-160; a left
                // end before column 0 is clamped to column 0, :153-154)
#pragma unroll
                for (int u = 0; u < kHSub; u++) {
                    const int xs = hx - kHLag + u;
                    if (!decltype(edge)::value || (xs >= 0 && xs < W)) {
                        const uint32_t e = LR[((kHSub * h + u - kHLag) & 31) * 32];
                        const int xsl = xs << 7;
                        const int il = imax(xsl - (int)(e & 0xffffu), 0);
                        const int ir = xsl + (int)(e >> 16);
                        // slot (column & 63) of the ring: the byte offset is (column << 7) & 0x1f80
                        const float pl = PR[(il & 0x1f80) >> 2];
                        const float pr = PR[(ir & 0x1f80) >> 2];
                        if (active) seg[(size_t)xs * D] = to_store<ST>(__fsub_rn(pr, pl));
                    }
                }
                uint32_t *LRh = LR + kHSub * h * 32;
#pragma unroll
                for (int u = 0; u < kHSub; u++) LRh[u * 32] = lv[u];
            };
            // a group whose segments are all inside the row needs no column checks
            auto run = [&](auto hc) {
                constexpr int h = decltype(hc)::value;
                const int g0 = x0 + kHSub * h;
                if (g0 >= kHLag && g0 + kHSub - 1 - kHLag < W) group(hc, std::false_type{});
                else group(hc, std::true_type{});
            };
            run(std::integral_constant<int, 0>{});
            run(std::integral_constant<int, 1>{});
            run(std::integral_constant<int, 2>{});
            run(std::integral_constant<int, 3>{});
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// vert: block per (view, column x, strip of rows).  Rows enter a shared ring 8
// at a time ("ticks", warp w ingesting row w of the tick); for every entry the
// ring holds the row segment and the row's pixel count l + r + 1, and the
// entry's vertical arms t | b << 8.  Each step a warp computes one output row
// y: it walks the rows of the reference pixel's own vertical arm (a superset of
// every disparity's arm) and adds a row's segment and count where the row lies
// in that disparity's arm [y - t, y + b], top to bottom
// (seq/CrossBasedAggregation.cpp:140-164); the average is the correctly rounded
// quotient (:166) and the winner the first strict minimum over d.
constexpr int kVertW = 8;
constexpr int kVertT = kVertW * 32;

// ring depth and first ticks: rts_vert_ring.h (shared with the CPU check of
// the ring arithmetic)

// The ring accumulators: where a row lies in a disparity's arm, its segment is
// added to the sum and its pixel count to the count, as predicated instructions
// (a branch per row and disparity would cost more than the two adds).
template <typename ST> struct VRing;
template <> struct VRing<float> {
    using E = uint2;   // {segment bits, row pixel count}
    using In = float;  // what the ingest loads from the segment volume
    struct Acc {
        float s;
        uint32_t c;
    };
    static __device__ __forceinline__ E make(float s, uint32_t cnt) { return make_uint2(__float_as_uint(s), cnt); }
    static __device__ __forceinline__ Acc zero() { return Acc{0.f, 0u}; }
    // the entry at shared address a + OFF (bytes)
    template <int OFF> static __device__ __forceinline__ E lds(uint32_t a) {
        E e;
        asm volatile("ld.shared.v2.u32 {%0, %1}, [%2+%3];" : "=r"(e.x), "=r"(e.y) : "r"(a), "n"(OFF));
        return e;
    }
    static __device__ __forceinline__ void add_if_bit(Acc &a, uint32_t m, uint32_t bit, E e) {
        asm("{\n\t.reg .pred p;\n\t.reg .b32 t;\n\tand.b32 t, %2, %3;\n\tsetp.ne.u32 p, t, 0;\n\t"
            "@p add.rn.f32 %0, %0, %4;\n\t@p add.u32 %1, %1, %5;\n\t}"
            : "+f"(a.s), "+r"(a.c)
            : "r"(m), "r"(bit), "f"(__uint_as_float(e.x)), "r"(e.y));
    }
    static __device__ __forceinline__ void add_if_lt(Acc &a, uint32_t x, uint32_t y, E e) {
        asm("{\n\t.reg .pred p;\n\tsetp.lo.u32 p, %2, %3;\n\t@p add.rn.f32 %0, %0, %4;\n\t@p add.u32 %1, %1, %5;\n\t}"
            : "+f"(a.s), "+r"(a.c)
            : "r"(x), "r"(y), "f"(__uint_as_float(e.x)), "r"(e.y));
    }
    static __device__ __forceinline__ float sum(Acc a) { return a.s; }
    static __device__ __forceinline__ uint32_t cnt(Acc a) { return a.c; }
};
template <> struct VRing<__half> {
    // count in the low half (sums of whole words keep it exact below 2^16),
    // f16 segment in the high half
    using E = uint32_t;
    using In = unsigned short;  // the f16 bits
    struct Acc {
        float s;
        uint32_t c;
    };
    static __device__ __forceinline__ E make(unsigned short s, uint32_t cnt) { return ((uint32_t)s << 16) | cnt; }
    static __device__ __forceinline__ Acc zero() { return Acc{0.f, 0u}; }
    template <int OFF> static __device__ __forceinline__ E lds(uint32_t a) {
        E e;
        asm volatile("ld.shared.u32 %0, [%1+%2];" : "=r"(e) : "r"(a), "n"(OFF));
        return e;
    }
    // the segment enters the f32 sum through the mixed-precision add (f16 operand
    // widened exactly, one rounding: the same result as converting, then adding)
    static __device__ __forceinline__ void add_if_bit(Acc &a, uint32_t m, uint32_t bit, E e) {
        asm("{\n\t.reg .pred p;\n\t.reg .b32 t;\n\t.reg .b16 lo, hi;\n\tand.b32 t, %2, %3;\n\t"
            "setp.ne.u32 p, t, 0;\n\tmov.b32 {lo, hi}, %4;\n\t"
            "@p add.rn.f32.f16 %0, hi, %0;\n\t@p add.u32 %1, %1, %4;\n\t}"
            : "+f"(a.s), "+r"(a.c)
            : "r"(m), "r"(bit), "r"(e));
    }
    static __device__ __forceinline__ void add_if_lt(Acc &a, uint32_t x, uint32_t y, E e) {
        asm("{\n\t.reg .pred p;\n\t.reg .b16 lo, hi;\n\tsetp.lo.u32 p, %2, %3;\n\tmov.b32 {lo, hi}, %4;\n\t"
            "@p add.rn.f32.f16 %0, hi, %0;\n\t@p add.u32 %1, %1, %4;\n\t}"
            : "+f"(a.s), "+r"(a.c)
            : "r"(x), "r"(y), "r"(e));
    }
    static __device__ __forceinline__ float sum(Acc a) { return a.s; }
    static __device__ __forceinline__ uint32_t cnt(Acc a) { return a.c & 0xffffu; }
};

template <> struct VRing<uint16_t> {
    // integer costs: segment << 12 | row pixel count in one word, and one 32-bit
    // add accumulates both (a cross's sums stay below 2^20 and its count below
    // 2^12); the sum is the exact integer the reference's float adds reach
    using E = uint32_t;
    using In = unsigned short;
    struct Acc {
        uint32_t v;
    };
    static __device__ __forceinline__ E make(unsigned short s, uint32_t cnt) { return ((uint32_t)s << 12) | cnt; }
    static __device__ __forceinline__ Acc zero() { return Acc{0u}; }
    template <int OFF> static __device__ __forceinline__ E lds(uint32_t a) {
        E e;
        asm volatile("ld.shared.u32 %0, [%1+%2];" : "=r"(e) : "r"(a), "n"(OFF));
        return e;
    }
    static __device__ __forceinline__ void add_if_bit(Acc &a, uint32_t m, uint32_t bit, E e) {
        asm("{\n\t.reg .pred p;\n\t.reg .b32 t;\n\tand.b32 t, %1, %2;\n\tsetp.ne.u32 p, t, 0;\n\t"
            "@p add.u32 %0, %0, %3;\n\t}"
            : "+r"(a.v)
            : "r"(m), "r"(bit), "r"(e));
    }
    static __device__ __forceinline__ void add_if_lt(Acc &a, uint32_t x, uint32_t y, E e) {
        asm("{\n\t.reg .pred p;\n\tsetp.lo.u32 p, %1, %2;\n\t@p add.u32 %0, %0, %3;\n\t}"
            : "+r"(a.v)
            : "r"(x), "r"(y), "r"(e));
    }
    static __device__ __forceinline__ float sum(Acc a) { return __uint2float_rn(a.v >> 12); }
    static __device__ __forceinline__ uint32_t cnt(Acc a) { return a.v & 0xfffu; }
};

// One item (column x, rows y0 .. y1-1) with NC 32-disparity chunks per lane;
// DM is the ring row stride (entries) of the launch.
template <typename ST, int NC, int DM, int POS>
__device__ __forceinline__ void vert_item(const ViewDesc &V, int x, int y0, int y1, int L, int DEP,
                                          const float *__restrict__ rcp, unsigned char *vsm) {
    using RG = VRing<ST>;
    using E = typename RG::E;
    using In = typename RG::In;
    E *ring = reinterpret_cast<E *>(vsm);                                                // [DEP][DM]
    uint16_t *inf = reinterpret_cast<uint16_t *>(vsm + (size_t)DEP * DM * sizeof(E));    // [DEP][DM]
    uint32_t *rinf = reinterpret_cast<uint32_t *>(inf + (size_t)DEP * DM);               // [DEP]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = V.W, H = V.H, D = V.D, mir = V.mirror;
    const int ra = imax(0, y0 - L), rb = imin(H, y1 + L);
    const int xsrc = mir ? W - 1 - x : x;
    // per disparity (shared): the target image column of column x
    int *tcs = reinterpret_cast<int *>(rinf + DEP);  // [DM]
    auto dok = [&](int c) { return 32 * c + lane < D; };
    // the view's pointers, read once (the loops below store to shared memory, which
    // the compiler might otherwise take to alias the view table)
    const In *__restrict__ segx = reinterpret_cast<const In *>(V.seg) + (size_t)x * D + lane;  // + r W D + 32 c
    const uint2 *__restrict__ arefx = V.aref + xsrc;  // + r W
    const uint2 *__restrict__ atar = V.atar;
    uint16_t *__restrict__ rawx = V.raw + x;  // + y W
    int *__restrict__ rowl = V.row_last;
    const size_t segrow = (size_t)W * D;
    const int nticks = (rb - ra + 7) >> 3;
    // one tick's loads for this warp's row, in flight while the previous tick is used
    In pseg[NC];
    uint2 ptar[NC], pref;
    auto load_tick = [&](int i) {
        const int r = ra + 8 * i + warp;
        if (r < rb) {
            const uint2 *arow = atar + (size_t)r * W;
            pref = arefx[(size_t)r * W];
#pragma unroll
            for (int c = 0; c < NC; c++) {
                if (dok(c)) pseg[c] = segx[(size_t)r * segrow + 32 * c];
                ptar[c] = arow[tcs[32 * c + lane]];
            }
        }
    };
    int tslot = 0;  // ring slot of the next tick's first row
    // tick i into the ring, then the loads of tick i + 1 (used by the next step)
    auto ingest = [&](int i) {
        const int r = ra + 8 * i + warp;
        if (r < rb) {
            const int slot = tslot + warp;
            E *er = ring + slot * DM + lane;
            uint16_t *ir = inf + slot * DM + lane;
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const uint32_t m = __vminu2(pref.x, ptar[c].x);   // l | r << 16
                const uint32_t cnt = __dp2a_lo(m, 0x0101u, 1u);   // l + r + 1
                const uint32_t tb = __vminu2(pref.y, ptar[c].y);  // t | b << 16
                // t | (t + b + 1) << 8: the start and length of the arm; 0 for no disparity
                const uint32_t tw = __dp2a_lo(tb, 0x0101u, 1u) << 8 | (tb & 0xffu);
                if (dok(c)) er[32 * c] = RG::make(pseg[c], cnt);
                ir[32 * c] = dok(c) ? (uint16_t)tw : (uint16_t)0;
            }
            if (lane == 0) rinf[slot] = __byte_perm(pref.y, 0, 0x4420);
        }
        tslot += 8;
        if (tslot == DEP) tslot = 0;
        if (i + 1 < nticks) load_tick(i + 1);
    };
    __syncthreads();  // the previous item's readers are done with the ring
    for (int d = threadIdx.x; d < DM; d += kVertT) {
        int xt = x - (d < D ? d : 0);
        if (xt < 0) xt += W;  // seq/PixelBasedCost.cpp:19-20 (D <= W)
        tcs[d] = mir ? W - 1 - xt : xt;
    }
    __syncthreads();
    load_tick(0);
    const int T0 = vert_first_ticks(y0, ra, L);  // ticks the first step needs
    int i = 0;
    for (; i < T0 - 1; i++) ingest(i);
    const int nsteps = (y1 - y0 + 7) >> 3;
    int sbase = y0 - ra;  // ring slot of row y0 + 8s (< DEP)
    for (int s = 0; s < nsteps; s++, i++) {
        ingest(i);
        __syncthreads();
        const int y = y0 + 8 * s + warp;
        if (y < y1) {
            int sy = sbase + warp;
            if (sy >= DEP) sy -= DEP;
            const uint32_t ri = rinf[sy];
            const int tr = ri & 0xff, br = ri >> 8;
            const int K = tr + br + 1;
            int slot = sy - tr;
            if (slot < 0) slot += DEP;
            // per disparity: its arm starts at row y - t, counted from y - tr (lo), and has
            // t + b + 1 rows (len; 0 where there is no disparity)
            const uint16_t *infy = inf + sy * DM + lane;
            auto lo = [&](int c) { return tr - (int)(infy[32 * c] & 0xff); };
            auto len = [&](int c) { return (int)(infy[32 * c] >> 8); };
            typename RG::Acc acc[NC];
#pragma unroll
            for (int c = 0; c < NC; c++) acc[c] = RG::zero();
            // rows y - tr .. y + br, top to bottom, wrapping once in the ring
            if (K <= 31) {
                // blocks of two rows from the even slot at or below the first row (DEP is
                // even, so a block never straddles the ring's wrap); the bits of the rows of
                // each disparity's arm, counted from that slot, in msk
                const int off = slot & 1;
                uint32_t msk[NC];
#pragma unroll
                for (int c = 0; c < NC; c++)
                    asm("bmsk.clamp.b32 %0, %1, %2;" : "=r"(msk[c]) : "r"(lo(c) + off), "r"(len(c)));
                // 32-bit shared addresses, entries at immediate offsets
                constexpr int ES = (int)sizeof(E), RS = DM * ES;  // entry, ring row bytes
                const uint32_t r0 = (uint32_t)__cvta_generic_to_shared(ring + lane);
                const uint32_t rend = r0 + (uint32_t)(DEP * RS);
                uint32_t ra = r0 + (uint32_t)((slot - off) * RS);
                const int nb = (K + off + 1) >> 1;
                for (int bk = 0; bk < nb; bk++) {
                    auto chunk = [&](auto cc) {
                        constexpr int c = decltype(cc)::value;
                        const E e0 = RG::template lds<32 * c * ES>(ra);
                        const E e1 = RG::template lds<RS + 32 * c * ES>(ra);
                        RG::add_if_bit(acc[c], msk[c], 1u, e0);
                        RG::add_if_bit(acc[c], msk[c], 2u, e1);
                        msk[c] >>= 2;
                    };
                    chunk(std::integral_constant<int, 0>{});
                    if constexpr (NC > 1) chunk(std::integral_constant<int, 1>{});
                    if constexpr (NC > 2) {
                        chunk(std::integral_constant<int, 2>{});
                        chunk(std::integral_constant<int, 3>{});
                    }
                    if constexpr (NC > 4) {
                        chunk(std::integral_constant<int, 4>{});
                        chunk(std::integral_constant<int, 5>{});
                        chunk(std::integral_constant<int, 6>{});
                        chunk(std::integral_constant<int, 7>{});
                    }
                    ra += 2 * RS;
                    if (ra == rend) ra = r0;
                }
            } else {
                for (int k = 0; k < K; k++) {
                    const E *rp = ring + slot * DM + lane;
#pragma unroll
                    for (int c = 0; c < NC; c++) {
                        const E e = rp[32 * c];
                        // k in [lo, lo + len): k - lo < len as unsigned
                        RG::add_if_lt(acc[c], (uint32_t)(k - lo(c)), (uint32_t)len(c), e);
                    }
                    if (++slot == DEP) slot = 0;
                }
            }
            uint32_t best_key = 0xffffffffu;
            int best_d = 0;
#pragma unroll
            for (int c = 0; c < NC; c++) {
                if (dok(c)) {
                    const float sm = RG::sum(acc[c]);
                    const uint32_t cn = RG::cnt(acc[c]);
                    const float cf = (float)cn;
                    uint32_t key;
                    if constexpr (POS) {
                        // sums of non-negative costs: the correctly rounded quotient by
                        // Markstein's correction from a correctly rounded reciprocal
                        // (Markstein 1990; exact residual by FMA), and the bits of a
                        // non-negative float order like the float
                        const float rcb = __ldg(rcp + cn);
                        const float q0 = __fmul_rn(sm, rcb);
                        const float rr = __fmaf_rn(-cf, q0, sm);
                        key = __float_as_uint(__fmaf_rn(rr, rcb, q0));
                    } else {
                        key = order_key(__fdiv_rn(sm, cf));
                    }
                    if (key < best_key) {  // strict: the lowest d keeps ties
                        best_key = key;
                        best_d = 32 * c + lane;
                    }
                }
            }
            const uint32_t m = __reduce_min_sync(0xffffffffu, best_key);
            const uint32_t bd = __reduce_min_sync(0xffffffffu, best_key == m ? (uint32_t)best_d : 0xffffu);
            if (lane == 0) {
                const bool found = bd != 0;  // some d >= 1 strictly below cost[0]
                rawx[(size_t)y * W] = found ? (uint16_t)(0x100 | bd) : (uint16_t)0;
                if (found) atomicMax(rowl + y, x);
            }
        }
        sbase += 8;
        if (sbase >= DEP) sbase -= DEP;
    }
}

template <typename ST, int NCH, int POS>
__global__ void __launch_bounds__(kVertT, NCH <= 4 ? 2 : 1)
    k_vert_views(ViewTable t, int L, int R, int DEP, const float *__restrict__ rcp) {
    constexpr int DM = 32 * NCH;  // ring row stride in entries
    extern __shared__ __align__(16) unsigned char vsm[];
    const int nv = t.nviews;
    const int *off = t.off + ST_VERT * (nv + 1);
    for (int item = blockIdx.x; item < t.total[ST_VERT]; item += gridDim.x) {
        const int v = find_view(off, nv, item);
        const ViewDesc &V = t.views[v];
        const int H = V.H;
        const int strips = (H + R - 1) / R;
        const int local = item - __ldg(off + v);
        const int x = local / strips, strip = local - x * strips;
        const int y0 = strip * R, y1 = imin(H, y0 + R);
        const int nch = (V.D + 31) >> 5;
        if (nch <= 1 || NCH == 1) vert_item<ST, 1, DM, POS>(V, x, y0, y1, L, DEP, rcp, vsm);
        else if (nch <= 2 || NCH == 2) vert_item<ST, (NCH >= 2 ? 2 : 1), DM, POS>(V, x, y0, y1, L, DEP, rcp, vsm);
        else if (nch <= 4 || NCH == 4) vert_item<ST, (NCH >= 4 ? 4 : 1), DM, POS>(V, x, y0, y1, L, DEP, rcp, vsm);
        else vert_item<ST, NCH, DM, POS>(V, x, y0, y1, L, DEP, rcp, vsm);
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
int stage_items(int stage, const ViewDesc &v, int vert_rows) {
    switch (stage) {
    case ST_PREP: return v.prep ? 2 * ((v.W + kPrepTW - 1) / kPrepTW) * ((v.H + kPrepTH - 1) / kPrepTH) : 0;
    case ST_HSEG: return v.H * ((v.D + 31) / 32);
    case ST_VERT: return v.W * ((v.H + vert_rows - 1) / vert_rows);
    case ST_FILL: return v.H;
    case ST_CC: return v.H;
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

template <typename K> static int resident_blocks(K kern, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem) != cudaSuccess || n < 1) n = 1;
    return n;
}

static bool mode1(const rts_params &p) {
    // AD (truncated, seq/Main.cpp:183-186) with an integral truncation, or rank
    // differences, combined with census: integer costs through one host table
    const bool ad = p.cost1 == RTS_COST_AD && p.ad_trunc >= 0.f && p.ad_trunc < (float)kCombineLut &&
                    p.ad_trunc == floorf(p.ad_trunc);
    return (ad || (p.cost1 == RTS_COST_RANK && p.rank_rad <= 16)) && p.cost2 == RTS_COST_CENSUS;
}
// the largest first-cost value of the table path (its truncation)
static int mode1_smax(const rts_params &p) { return p.cost1 == RTS_COST_RANK ? 255 : (int)p.ad_trunc; }

// The largest cost of a configuration whose costs are all integers (census
// alone, or truncated AD alone with an integral truncation), else -1.
static int int_cost_max(const rts_params &p) {
    if (p.cost2 != RTS_COST_NONE) return -1;
    if (p.cost1 == RTS_COST_CENSUS) return (2 * p.census_hrad + 1) * (2 * p.census_wrad + 1);
    if (p.cost1 == RTS_COST_AD && p.aggr == RTS_AGGR_CROSS && p.ad_trunc >= 0.f && p.ad_trunc <= 765.f &&
        p.ad_trunc == floorf(p.ad_trunc))
        return (int)p.ad_trunc;  // seq/Main.cpp:183-186: AD is truncated in the cross-based runs
    return -1;
}

int cross_seg_kind(const rts_params &p, int max_w) {
    const int m = int_cost_max(p);
    const long cross = (long)(2 * p.cross_arm + 1) * (2 * p.cross_arm + 1);
    // exact integers all the way: row prefix sums below 2^24 (float), a cross's
    // sum below 2^20 and its pixel count below 2^12 (the packed vertical adds)
    if (m >= 0 && cross_record_costs(p) && (long)m * cross < (1L << 20) && cross < 4096 &&
        (long)max_w * m < (1L << 24))
        return 2;
    return p.precision == RTS_PREC_F16 ? 1 : 0;
}

bool cross_record_costs(const rts_params &p) {
    if (!mode1(p) && !fast_costs(p)) return false;
    const bool census = p.cost1 == RTS_COST_CENSUS || p.cost2 == RTS_COST_CENSUS;
    return !census || (2 * p.census_hrad + 1) * (2 * p.census_wrad + 1) <= 64;
}

rts_status cross_tables(rts_ctx *c, const rts_params &p) {
    const float *t;
    if (p.cost2 != RTS_COST_NONE) {
        const float *t2;
        RTS_TRY(combine_luts(c, p.lambda1, p.lambda2, &t, &t2));
    }
    RTS_TRY(recip_table(c, &t));
    return RTS_OK;
}

rts_status launch_cross_views(rts_ctx *c, const rts_params &p, const ViewTable &t, int segk, int has_vol, int gray,
                              int max_d, const CrossTune &tune, int *row_last_all, size_t row_last_count) {
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
    const int mode = has_vol ? 0 : mode1(p) ? 1 : 2;
    const float *rcp = nullptr;
    if (mode == 1) cfg.itrunc = mode1_smax(p);
    if (p.cost2 != RTS_COST_NONE) RTS_TRY(combine_luts(c, p.lambda1, p.lambda2, &cfg.lut1, &cfg.lut2));
    RTS_TRY(recip_table(c, &rcp));
    const bool rank = mode == 1 && p.cost1 == RTS_COST_RANK;
    // record colour word: 2 rank, 1 gray byte, 0 packed RGB
    const int grayrec = rank ? 2 : (mode == 1 && gray) ? 1 : 0;
    cudaStream_t s = c->stream;
    const int sms = num_sms();
    auto grid = [&](int items, int per_block, int per_sm) {
        const long need = ((long)items + per_block - 1) / per_block;
        const long cap = tune.persistent ? (long)sms * per_sm : need;
        return (unsigned)(need < cap ? (need > 0 ? need : 1) : cap);
    };
    const int L = p.cross_arm;
    RTS_CU(c, cudaMemsetAsync(row_last_all, 0xff, row_last_count * sizeof(int), s));
    const bool want_code = !has_vol && (p.cost1 == RTS_COST_CENSUS || p.cost2 == RTS_COST_CENSUS);
    if (t.total[ST_PREP] > 0) {
        StageScope sc(c, "prep");
        const int hr = want_code ? p.census_hrad : 0, wr = want_code ? p.census_wrad : 0;
        const int rk = rank ? p.rank_rad : -1;
        const int gr = std::max(hr, std::max(rk, 0)), gc = std::max(wr, std::max(rk, 0));
        const size_t smem = prep_smem(gr, gc, L);
        auto go = [&](auto kern) -> rts_status {
            RTS_TRY(set_smem(c, kern, smem, "prep_views"));
            kern<<<grid(t.total[ST_PREP], 1, resident_blocks(kern, kPrepT, smem)), kPrepT, smem, s>>>(
                t, hr, wr, L, p.cross_tau, want_code ? 1 : 0, rk, gr, gc);
            return RTS_OK;
        };
        if (grayrec == 1) RTS_TRY(go(k_prep_views<1>));
        else RTS_TRY(go(k_prep_views<0>));
        count_launch(c);
    }
    {
        StageScope sc(c, "cross_hseg");
        const unsigned g = grid(t.total[ST_HSEG], kHsegW, tune.grid_mult);
        auto go = [&](auto kern) { kern<<<g, kHsegW * 32, 0, s>>>(t, cfg); };
        if (segk == 2) {
            // integer costs: census alone, or truncated AD alone
            if (p.cost1 == RTS_COST_CENSUS) go(k_hseg_views<uint16_t, 3, 0>);
            else go(k_hseg_views<uint16_t, 4, 0>);
        } else if (segk == 1) {
            if (mode == 0) go(k_hseg_views<__half, 0, 0>);
            else if (mode == 1 && grayrec == 2) go(k_hseg_views<__half, 1, 2>);
            else if (mode == 1 && grayrec == 1) go(k_hseg_views<__half, 1, 1>);
            else if (mode == 1) go(k_hseg_views<__half, 1, 0>);
            else go(k_hseg_views<__half, 2, 0>);
        } else {
            if (mode == 0) go(k_hseg_views<float, 0, 0>);
            else if (mode == 1 && grayrec == 2) go(k_hseg_views<float, 1, 2>);
            else if (mode == 1 && grayrec == 1) go(k_hseg_views<float, 1, 1>);
            else if (mode == 1) go(k_hseg_views<float, 1, 0>);
            else go(k_hseg_views<float, 2, 0>);
        }
        count_launch(c);
    }
    {
        StageScope sc(c, "cross_vert_wta");
        const int DEP = vert_depth(L);
        const int nch = (max_d + 31) / 32;
        const int NCH = nch <= 1 ? 1 : nch <= 2 ? 2 : nch <= 4 ? 4 : 8;
        // ring {segment, count} + arm words + reference arm words + target columns
        const size_t DMb = (size_t)32 * NCH;
        const size_t smem = (size_t)DEP * DMb * ((segk ? 4 : 8) + 2) + (size_t)DEP * 4 + DMb * 4;
        const int R = tune.vert_rows;
        rts_status vs = RTS_OK;
        auto go = [&](auto kern) {
            vs = set_smem(c, kern, smem, "vert_views");
            if (vs != RTS_OK) return;
            kern<<<grid(t.total[ST_VERT], 1, resident_blocks(kern, kVertT, smem)), kVertT, smem, s>>>(t, L, R, DEP,
                                                                                                   rcp);
        };
        // non-negative costs take the fast exact division: every cost made from records,
        // and every precomputed volume but NCC's (AD, rank and LoG differences, Hamming
        // distances and their CombineCost terms 1 - exp(-v / lambda) are >= 0)
        const bool pos = mode != 0 || (p.cost1 != RTS_COST_NCC && p.cost2 != RTS_COST_NCC);
#define RTS_VERT(ST, N)                                   \
    do {                                                  \
        if (!pos) go(k_vert_views<ST, N, 0>);             \
        else go(k_vert_views<ST, N, 1>);                  \
    } while (0)
        if (segk == 2) {
            if (NCH == 1) go(k_vert_views<uint16_t, 1, 1>);
            else if (NCH == 2) go(k_vert_views<uint16_t, 2, 1>);
            else if (NCH == 4) go(k_vert_views<uint16_t, 4, 1>);
            else go(k_vert_views<uint16_t, 8, 1>);
        } else if (segk == 1) {
            if (NCH == 1) RTS_VERT(__half, 1);
            else if (NCH == 2) RTS_VERT(__half, 2);
            else if (NCH == 4) RTS_VERT(__half, 4);
            else RTS_VERT(__half, 8);
        } else {
            if (NCH == 1) RTS_VERT(float, 1);
            else if (NCH == 2) RTS_VERT(float, 2);
            else if (NCH == 4) RTS_VERT(float, 4);
            else RTS_VERT(float, 8);
        }
#undef RTS_VERT
        RTS_TRY(vs);
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
