/*
 * rts_oracle.c -- CPU oracle (plain C restatement of rtstereo seq/ sources).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py, as the checker or the timed CPU baseline.  The
 * product (rtstereo_gb300) never links or calls it.
 *
 * Parity pin: tests/test_oracle_vs_reference.py checks every function here
 * bit-for-bit against the reference's own seq/ sources compiled from source into
 * oracle/_ref/ (where the reference is present), and tests/test_oracle_golden.py
 * checks it against the committed fixtures made from that build.
 *
 * Build with -ffp-contract=off: the reference (g++ -O2, x86-64) fuses no
 * multiply-add, and on aarch64 gcc would otherwise contract a*b+c.
 */
#include "rts_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Output rows of the out-of-place functions are independent, so their row
 * loops may run on several host threads (OpenMP, when the build has it): every
 * entry is still computed by one thread with the same operations in the same
 * order, so the results do not depend on the thread count.  The in-place
 * recurrences (orc_box_inplace, orc_aw_r2l, orc_disp_refinement) and the WTA
 * winner carry stay serial. */
#ifdef _OPENMP
#include <omp.h>
#define ORC_PRAGMA(x) _Pragma(#x)
#define ORC_PAR ORC_PRAGMA(omp parallel for schedule(dynamic, 1))
#define ORC_PAR_IF(c) ORC_PRAGMA(omp parallel for schedule(dynamic, 1) if (c))
#define ORC_PAR_FLAT ORC_PRAGMA(omp parallel for schedule(static))
#define ORC_PAR_PIXELS ORC_PRAGMA(omp parallel for collapse(2) schedule(dynamic, 16))
#else
#define ORC_PAR_FLAT
#define ORC_PAR_PIXELS
#define ORC_PAR
#define ORC_PAR_IF(c)
#endif

void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
    (void)n;
#endif
}

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

const float orc_log5x5[25] = {
    0.0239f, 0.046f,   0.0499f,  0.046f,   0.0239f,
    0.046f,  0.0061f, -0.0923f,  0.0061f,  0.046f,
    0.0499f, -0.0923f, -0.3182f, -0.0923f, 0.0499f,
    0.046f,  0.0061f, -0.0923f,  0.0061f,  0.046f,
    0.0239f, 0.046f,   0.0499f,  0.046f,   0.0239f};

/* single wrap of an index that is at most one period outside [0, n) */
static inline int wrap1(int i, int n) {
    if (i < 0) return i + n;
    if (i >= n) return i - n;
    return i;
}

static inline int iabs(int v) { return v < 0 ? -v : v; }

/* target column for disparity d: L2R x-d (+W if <0), R2L x+d (-W if >=W).
 * seq/PixelBasedCost.cpp:19-20 (L2R) and :32-33 (R2L). */
static inline int tar_col(int x, int d, int W, int dir) {
    int xt = (dir == ORC_L2R) ? x - d : x + d;
    if (dir == ORC_L2R) { if (xt < 0) xt += W; }
    else { if (xt >= W) xt -= W; }
    return xt;
}

/* seq/PixelBasedCost.cpp:13-37 pixelBasedL2R / pixelBasedR2L */
void orc_ad_gray(const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int dir) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                int xt = tar_col(x, d, W, dir);
                cost[d + (long)D * p] = (float)iabs((int)ref[p] - (int)tar[(long)y * W + xt]);
            }
        }
}

/* seq/PixelBasedCost.cpp:39-69 pixelBasedCostL2R_Float / pixelBasedCostR2L_Float */
void orc_ad_float(const float *ref, const float *tar, float *cost, int D, int H, int W, int dir) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                int xt = tar_col(x, d, W, dir);
                float r = ref[p] - tar[(long)y * W + xt];
                if (r < 0) r = -r;
                cost[d + (long)D * p] = r;
            }
        }
}

/* seq/PixelBasedCost.cpp:72-158: the four colour variants.  norm!=0 scales by
 * (float)1/(float)3 after the (optional) truncation min(sad, trunc). */
void orc_ad_color(const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W,
                  int dir, int use_trunc, float trunc, int norm) {
    const float third = (float)1 / (float)3;
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                long q = (long)y * W + tar_col(x, d, W, dir);
                int sad = iabs((int)ref[3 * p] - (int)tar[3 * q]) +
                          iabs((int)ref[3 * p + 1] - (int)tar[3 * q + 1]) +
                          iabs((int)ref[3 * p + 2] - (int)tar[3 * q + 2]);
                float v;
                if (use_trunc) v = ((float)sad > trunc) ? trunc : (float)sad;
                else v = (float)sad;
                if (norm) v = third * v;
                cost[d + (long)D * p] = v;
            }
        }
}

/* seq/CensusTransform.cpp:11-37: bit (y'+hrad)*(2wrad+1)+(x'+wrad) is 1 iff
 * centre > neighbour (strict), neighbours wrap around both borders. */
void orc_census(const uint8_t *img, uint8_t *bits, int hrad, int wrad, int H, int W) {
    int bw = 2 * wrad + 1, nb = (2 * hrad + 1) * bw;
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            uint8_t c = img[p];
            for (int dy = -hrad; dy <= hrad; dy++) {
                int yy = wrap1(y + dy, H);
                for (int dx = -wrad; dx <= wrad; dx++) {
                    int xx = wrap1(x + dx, W);
                    bits[(dy + hrad) * bw + (dx + wrad) + (long)nb * p] = (c > img[(long)yy * W + xx]) ? 1 : 0;
                }
            }
        }
}

/* seq/CensusTransform.cpp:39-62: number of differing bits between the ref pixel
 * and the target pixel x-d (wrapped). */
void orc_hamming(const uint8_t *bref, const uint8_t *btar, float *cost, int hrad, int wrad,
                 int H, int W, int D) {
    int nb = (2 * hrad + 1) * (2 * wrad + 1);
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                long q = (long)y * W + tar_col(x, d, W, ORC_L2R);
                int cnt = 0;
                for (int k = 0; k < nb; k++)
                    cnt += ((bref[k + (long)nb * p] != 0) != (btar[k + (long)nb * q] != 0));
                cost[d + (long)D * p] = (float)cnt;
            }
        }
}

/* seq/RankFilter.cpp:11-35: 1 + #{neighbours strictly darker than the centre}
 * over a (2rad+1)^2 wrapped window, stored as unsigned char (wraps above 255). */
void orc_rank(const uint8_t *img, uint8_t *out, int rad, int H, int W) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            int cnt = 1;
            uint8_t c = img[p];
            for (int dy = -rad; dy <= rad; dy++) {
                int yy = wrap1(y + dy, H);
                for (int dx = -rad; dx <= rad; dx++) {
                    int xx = wrap1(x + dx, W);
                    if (img[(long)yy * W + xx] < c) cnt++;
                }
            }
            out[p] = (uint8_t)cnt;
        }
}

/* seq/ConvolveImage.cpp:11-35: raster-order sum of rounded float products,
 * then |.| and min(.,255). */
void orc_convolve(const uint8_t *img, float *out, const float *mask, int H, int W, int hrad, int wrad) {
    int mw = 2 * wrad + 1;
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            float acc = 0;
            for (int dy = -hrad; dy <= hrad; dy++) {
                int yy = wrap1(y + dy, H);
                for (int dx = -wrad; dx <= wrad; dx++) {
                    int xx = wrap1(x + dx, W);
                    float prod = (float)img[(long)yy * W + xx] * mask[(dy + hrad) * mw + (dx + wrad)];
                    acc = acc + prod;
                }
            }
            acc = (acc > 0) ? acc : -acc;
            out[(long)y * W + x] = (acc > 255) ? 255 : acc;
        }
}

/* seq/NCCDisparity.cpp:11-73.  nom = sum (r-mr)(t-mt); den = sqrt(sum
 * (r-mr)^2 (t-mt)^2) (the reference's non-standard denominator, :66,69);
 * the cell is left unwritten when den == 0 (:70-71). */
void orc_ncc(const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int hrad, int wrad) {
    int area = (2 * hrad + 1) * (2 * wrad + 1);
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            float mr = 0;
            for (int dy = -hrad; dy <= hrad; dy++) {
                int yy = wrap1(y + dy, H);
                for (int dx = -wrad; dx <= wrad; dx++)
                    mr = mr + (float)ref[(long)yy * W + wrap1(x + dx, W)];
            }
            mr = mr / (float)area;
            for (int d = 0; d < D; d++) {
                float mt = 0;
                for (int dy = -hrad; dy <= hrad; dy++) {
                    int yy = wrap1(y + dy, H);
                    for (int dx = -wrad; dx <= wrad; dx++)
                        mt = mt + (float)tar[(long)yy * W + wrap1(x + dx - d, W)];
                }
                mt = mt / (float)area;
                float nom = 0, den = 0;
                for (int dy = -hrad; dy <= hrad; dy++) {
                    int yy = wrap1(y + dy, H);
                    for (int dx = -wrad; dx <= wrad; dx++) {
                        float rv = (float)ref[(long)yy * W + wrap1(x + dx, W)] - mr;
                        float tv = (float)tar[(long)yy * W + wrap1(x + dx - d, W)] - mt;
                        float rt = rv * tv;
                        nom = nom + rt;
                        float q = rv * rv;
                        q = q * tv;
                        q = q * tv;
                        den = den + q;
                    }
                }
                den = sqrtf(den);
                if (den != 0) cost[d + (long)D * p] = nom / den;
            }
        }
}

/* seq/CombineCost.cpp:11-25: c1 <- (1 - expf(-c1/l1)) + (1 - expf(-c2/l2)). */
void orc_combine(float *c1, const float *c2, float lambda1, float lambda2, int H, int W, int D) {
    long n = (long)H * W * D;
    ORC_PAR_FLAT
    for (long i = 0; i < n; i++) {
        float a = c1[i], b = c2[i];
        a = 1 - expf(-a / lambda1);
        b = 1 - expf(-b / lambda2);
        c1[i] = a + b;
    }
}

/* seq/ConstBlockAggregation.cpp:11-34 literally: in place, so later windows
 * read already-averaged neighbours. */
void orc_box_inplace(float *cost, int H, int W, int D, int rad) {
    int area = (2 * rad + 1) * (2 * rad + 1);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int d = 0; d < D; d++) {
                float s = 0;
                for (int dy = -rad; dy <= rad; dy++) {
                    int yy = wrap1(y + dy, H);
                    for (int dx = -rad; dx <= rad; dx++) {
                        int xx = wrap1(x + dx, W);
                        s = s + cost[d + (long)D * (xx + (long)W * yy)];
                    }
                }
                cost[d + (long)D * (x + (long)W * y)] = s / (float)area;
            }
}

/* Out-of-place form of seq/ConstBlockAggregation.cpp:15-31 (same y-outer,
 * x-inner summation order and wrap indices, reading from an unmodified input).
 * This is the contract of the GPU machine aggregation. */
void orc_box(const float *cost, float *out, int H, int W, int D, int rad) {
    int area = (2 * rad + 1) * (2 * rad + 1);
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int d = 0; d < D; d++) {
                float s = 0;
                for (int dy = -rad; dy <= rad; dy++) {
                    int yy = wrap1(y + dy, H);
                    for (int dx = -rad; dx <= rad; dx++) {
                        int xx = wrap1(x + dx, W);
                        s = s + cost[d + (long)D * (xx + (long)W * yy)];
                    }
                }
                out[d + (long)D * (x + (long)W * y)] = s / (float)area;
            }
}

/* max over the three channels of |a_c - b_c| (seq/CrossBasedAggregation.cpp:30-31) */
static inline int chan_delta(const uint8_t *a, const uint8_t *b) {
    int m = iabs((int)a[1] - (int)b[1]);
    int r = iabs((int)a[2] - (int)b[2]);
    if (r > m) m = r;
    int g = iabs((int)a[0] - (int)b[0]);
    if (g > m) m = g;
    return m;
}

/* One arm of seq/CrossBasedAggregation.cpp:12-100 (calc_x_range/calc_y_range):
 * step outward while the last visited pixel differs by < tau in every channel
 * and the arm is shorter than arm_len; the first failing pixel is included;
 * the arm stops at the image edge. */
static int arm_length(const uint8_t *rgb, long centre, long step, int room, int arm_len, int tau) {
    int len = 0, delta = 0;
    while (delta < tau && len < arm_len && len < room) {
        len++;
        delta = chan_delta(rgb + 3 * centre, rgb + 3 * (centre + step * len));
    }
    return len;
}

/* OpenCV medianBlur (opencl/Main.cpp:342-343; OpenCV documents replicated
 * borders for it): every channel separately, the window's values sorted by
 * insertion and the middle one taken. */
void orc_median(const uint8_t *img, uint8_t *out, int H, int W, int ch, int k) {
    int r = k / 2, n = k * k;
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int c = 0; c < ch; c++) {
                uint8_t v[225];
                int m = 0;
                for (int dy = -r; dy <= r; dy++)
                    for (int dx = -r; dx <= r; dx++) {
                        int yy = y + dy < 0 ? 0 : y + dy >= H ? H - 1 : y + dy;
                        int xx = x + dx < 0 ? 0 : x + dx >= W ? W - 1 : x + dx;
                        uint8_t a = img[((long)yy * W + xx) * ch + c];
                        int i = m++;
                        while (i > 0 && v[i - 1] > a) { v[i] = v[i - 1]; i--; }
                        v[i] = a;
                    }
                out[((long)y * W + x) * ch + c] = v[n / 2];
            }
}

/* seq/CrossBasedAggregation.cpp:102-115 findCross: horz[2p]=left, horz[2p+1]=right,
 * vert[2p]=top, vert[2p+1]=bottom. */
void orc_find_cross(const uint8_t *rgb, int *horz, int *vert, int H, int W, int arm_len, int tau) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            vert[2 * p] = arm_length(rgb, p, -(long)W, y, arm_len, tau);
            vert[2 * p + 1] = arm_length(rgb, p, (long)W, H - 1 - y, arm_len, tau);
            horz[2 * p] = arm_length(rgb, p, -1, x, arm_len, tau);
            horz[2 * p + 1] = arm_length(rgb, p, 1, W - 1 - x, arm_len, tau);
        }
}

/* seq/CrossBasedAggregation.cpp:117-125: in-place running sum along x per (y,d). */
void orc_prefix_h(float *cost, int H, int W, int D) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 1; x < W; x++)
            for (int d = 0; d < D; d++) {
                long i = d + (long)D * ((long)y * W + x);
                cost[i] = cost[i] + cost[i - D];
            }
}

/* seq/CrossBasedAggregation.cpp:127-169: per (x,y,d) the vertical arm is the
 * min of the ref arm at x and the target arm at x-d (wrapped); each row of it
 * contributes P[x+r] - P[x-l-1] with x-l-1 < 0 clamped to column 0 (that
 * pixel is then excluded from the sum but still counted, :151-162); the sum
 * of the rows in top-to-bottom order is divided by the pixel count. */
void orc_cross_aggr(const float *pre, float *out, const int *hr, const int *ht, const int *vr,
                    const int *vt, int H, int W, int D) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                int xt = tar_col(x, d, W, ORC_L2R);
                long q = (long)y * W + xt;
                int t = vr[2 * p] > vt[2 * q] ? vt[2 * q] : vr[2 * p];
                int b = vr[2 * p + 1] > vt[2 * q + 1] ? vt[2 * q + 1] : vr[2 * p + 1];
                float sum = 0;
                int cnt = 0;
                for (int dy = -t; dy <= b; dy++) {
                    int yy = y + dy;
                    if (yy < 0 || yy >= H) continue;
                    long pr = (long)yy * W + x, pt = (long)yy * W + xt;
                    int l = hr[2 * pr] > ht[2 * pt] ? ht[2 * pt] : hr[2 * pr];
                    int r = hr[2 * pr + 1] > ht[2 * pt + 1] ? ht[2 * pt + 1] : hr[2 * pr + 1];
                    int xl = x - l - 1, xr = x + r;
                    if (xl < 0) xl = 0;
                    else if (xr >= W) xr = W - 1;
                    if (xl >= 0 && xr < W) {
                        float seg = pre[d + (long)D * ((long)yy * W + xr)] - pre[d + (long)D * ((long)yy * W + xl)];
                        sum = sum + seg;
                        cnt += r + l + 1;
                    }
                }
                sum = sum / (float)cnt;
                out[d + (long)D * p] = sum;
            }
        }
}

/* seq/AdaptiveWeightAggregation.cpp:11-18: pw[k] = expf(-sqrtf(dy^2+dx^2)/gamma_p). */
void orc_prox_weight(float *pw, float gamma_p, int rad) {
    int k = 0;
    for (int dy = -rad; dy <= rad; dy++)
        for (int dx = -rad; dx <= rad; dx++) {
            float r = sqrtf((float)(dy * dy + dx * dx));
            pw[k++] = expf(-r / gamma_p);
        }
}

/* seq/AdaptiveWeightAggregation.cpp:19-24 calcEuclideanDist3P */
static inline float lab_dist(int l0, int l1, int a0, int a1, int b0, int b1) {
    float e0 = (float)l0 - (float)l1, e1 = (float)a0 - (float)a1, e2 = (float)b0 - (float)b1;
    float s = e0 * e0;
    s = s + e1 * e1;
    s = s + e2 * e2;
    return sqrtf(s);
}

/* seq/AdaptiveWeightAggregation.cpp:33-71: w[p][k] = pw[k]*expf(-|Lab(p)-Lab(q)|/gamma_s),
 * 0 where q falls outside the image (no wrap). */
void orc_compute_weights(float *w, const float *pw, const uint8_t *lab, float gamma_s, int H, int W, int rad) {
    orc_compute_weights_rows(w, pw, lab, gamma_s, H, W, rad, 0, H);
}

/* The weights of the pixels of rows y0 .. y0+nrows-1 only, into w[(y-y0)*W+x][k]. */
void orc_compute_weights_rows(float *w, const float *pw, const uint8_t *lab, float gamma_s, int H, int W, int rad,
                              int y0, int nrows) {
    int edge = 2 * rad + 1, area = edge * edge;
    ORC_PAR_PIXELS
    for (int y = y0; y < y0 + nrows; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x, pw_ = (long)(y - y0) * W + x;
            const uint8_t *c = lab + 3 * p;
            int k = 0;
            for (int dy = -rad; dy <= rad; dy++) {
                int yy = y + dy;
                for (int dx = -rad; dx <= rad; dx++, k++) {
                    int xx = x + dx;
                    float v = 0;
                    if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
                        const uint8_t *q = lab + 3 * ((long)yy * W + xx);
                        float dist = lab_dist(c[0], q[0], c[1], q[1], c[2], q[2]);
                        v = pw[k] * expf(-dist / gamma_s);
                    }
                    w[k + (long)area * pw_] = v;
                }
            }
        }
}

/* seq/AdaptiveWeightAggregation.cpp:73-111: out = sum_k wR[p][k] wT[p-d][k] C[q_k,d]
 * / sum_k wR wT; q_k wraps in x and y, the target pixel p-d wraps in x. */
void orc_aw_l2r(const float *wref, const float *wtar, const float *cost, float *out, int H, int W, int D, int rad) {
    orc_aw_l2r_rows(wref, wtar, cost, out, H, W, D, rad, 0, H);
}

/* Rows y0 .. y0+nrows-1 of orc_aw_l2r: the weights are those of
 * orc_compute_weights_rows over the same rows, `out` holds those rows, `cost`
 * is the whole volume. */
void orc_aw_l2r_rows(const float *wref, const float *wtar, const float *cost, float *out, int H, int W, int D,
                     int rad, int y0, int nrows) {
    int edge = 2 * rad + 1, area = edge * edge;
    ORC_PAR_PIXELS
    for (int y = y0; y < y0 + nrows; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)(y - y0) * W + x;
            for (int d = 0; d < D; d++) {
                long t = (long)(y - y0) * W + tar_col(x, d, W, ORC_L2R);
                float sw = 0, sc = 0;
                int k = 0;
                for (int dy = -rad; dy <= rad; dy++) {
                    int yy = wrap1(y + dy, H);
                    for (int dx = -rad; dx <= rad; dx++, k++) {
                        int xx = wrap1(x + dx, W);
                        float wgt = wref[k + (long)area * p] * wtar[k + (long)area * t];
                        sw = sw + wgt;
                        float cw = cost[d + (long)D * ((long)yy * W + xx)] * wgt;
                        sc = sc + cw;
                    }
                }
                out[d + (long)D * p] = sc / sw;
            }
        }
}

/* seq/AdaptiveWeightAggregation.cpp:113-150 calcAWCostR2L body: the weights
 * are taken at the window pixel (ref) and at the window pixel shifted by +d
 * (target, wrapped); reads src, writes dst (src == dst gives the reference's
 * in-place behaviour, where later windows see already-written cells). */
static void aw_r2l_core(const float *wref, const float *wtar, const float *src, float *dst,
                        int H, int W, int D, int rad) {
    int edge = 2 * rad + 1, area = edge * edge;
    ORC_PAR_IF(src != dst)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                float sw = 0, sc = 0;
                int k = 0;
                for (int dy = -rad; dy <= rad; dy++) {
                    int yy = wrap1(y + dy, H);
                    for (int dx = -rad; dx <= rad; dx++, k++) {
                        int xr = wrap1(x + dx, W);
                        int xt = wrap1(x + dx + d, W);
                        long pr = (long)yy * W + xr, pt = (long)yy * W + xt;
                        float wgt = wref[k + (long)area * pr] * wtar[k + (long)area * pt];
                        sw = sw + wgt;
                        float cw = src[d + (long)D * pr] * wgt;
                        sc = sc + cw;
                    }
                }
                dst[d + (long)D * p] = sc / sw;
            }
        }
}

void orc_aw_r2l(const float *wref, const float *wtar, float *cost, int H, int W, int D, int rad) {
    aw_r2l_core(wref, wtar, cost, cost, H, W, D, rad);
}

void orc_aw_r2l_oop(const float *wref, const float *wtar, const float *cost, float *out, int H, int W, int D, int rad) {
    aw_r2l_core(wref, wtar, cost, out, H, W, D, rad);
}

/* seq/WTA.cpp:10-39: first strict arg-min (argmax for NCC) over d >= 1 against
 * cost[0]; the winner variable is declared once per call, so a pixel with no
 * strictly better d >= 1 keeps the previous pixel's value (raster order). */
void orc_wta(const float *cost, uint8_t *win, int H, int W, int D, int argmax) {
    uint8_t disp = 0;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const float *c = cost + (long)D * ((long)y * W + x);
            float best = c[0];
            for (int d = 1; d < D; d++) {
                int better = argmax ? (c[d] > best) : (c[d] < best);
                if (better) { best = c[d]; disp = (uint8_t)d; }
            }
            win[(long)y * W + x] = disp;
        }
}

/* seq/CrossCheck.cpp:10-23: mask = (dref(x) == dtar(x - dref(x), wrapped)). */
void orc_cross_check(const uint8_t *dref, const uint8_t *dtar, uint8_t *mask, int H, int W) {
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            int v = dref[p];
            int xt = x - v;
            if (xt < 0) xt += W;
            mask[p] = (dtar[(long)y * W + xt] == v) ? 1 : 0;
        }
}

/* seq/CrossBasedAggregation.cpp:171-212 disp_refinement body: the mode of the
 * disparities in the cross region (rows y-top .. y+bottom-1, row segment
 * x-left .. x+right), strict first maximum over d < D.  Votes are read from
 * src; src == dst gives the reference's in-place behaviour (later pixels vote
 * with already-refined values). */
static void refine_core(const uint8_t *src, uint8_t *dst, const int *horz, const int *vert, int H, int W, int D) {
    ORC_PAR_IF(src != dst)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int hist[256];
            long p = (long)y * W + x;
            int t = vert[2 * p], b = vert[2 * p + 1];
            memset(hist, 0, sizeof(int) * 256);
            for (int dy = -t; dy < b; dy++) {
                int yy = y + dy;
                if (yy < 0 || yy >= H) continue;
                long pr = (long)yy * W + x;
                int xl = x - horz[2 * pr], xr = x + horz[2 * pr + 1];
                if (xl < 0) xl = 0;
                else if (xr >= W) xr = W - 1;
                for (int xx = xl; xx <= xr; xx++) hist[src[(long)yy * W + xx]]++;
            }
            int best = hist[0], arg = 0;
            for (int i = 1; i < D; i++)
                if (hist[i] > best) { best = hist[i]; arg = i; }
            dst[p] = (uint8_t)arg;
        }
}

void orc_disp_refinement(uint8_t *disp, const int *horz, const int *vert, int H, int W, int D) {
    refine_core(disp, disp, horz, vert, H, W, D);
}

void orc_disp_refinement_oop(const uint8_t *disp, uint8_t *out, const int *horz, const int *vert, int H, int W, int D) {
    refine_core(disp, out, horz, vert, H, W, D);
}

/* ------------------------------------------------------------------------- */
/* FP64 restatements                                                          */

void orc64_combine(const float *c1, const float *c2, double lambda1, double lambda2, long n, double *out) {
    for (long i = 0; i < n; i++)
        out[i] = (1.0 - exp(-(double)c1[i] / lambda1)) + (1.0 - exp(-(double)c2[i] / lambda2));
}

void orc64_aw_l2r(const uint8_t *labr, const uint8_t *labt, const float *cost, double *out,
                  int H, int W, int D, int rad, double gamma_s, double gamma_p) {
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                int xt = tar_col(x, d, W, ORC_L2R);
                long t = (long)y * W + xt;
                double sw = 0, sc = 0;
                for (int dy = -rad; dy <= rad; dy++) {
                    int yy = y + dy;
                    for (int dx = -rad; dx <= rad; dx++) {
                        double pw = exp(-sqrt((double)(dy * dy + dx * dx)) / gamma_p);
                        double wr = 0, wt = 0;
                        int xr = x + dx, xq = xt + dx;
                        if (yy >= 0 && yy < H && xr >= 0 && xr < W) {
                            const uint8_t *a = labr + 3 * p, *b = labr + 3 * ((long)yy * W + xr);
                            double e = sqrt((double)(a[0] - b[0]) * (a[0] - b[0]) + (double)(a[1] - b[1]) * (a[1] - b[1]) +
                                            (double)(a[2] - b[2]) * (a[2] - b[2]));
                            wr = pw * exp(-e / gamma_s);
                        }
                        if (yy >= 0 && yy < H && xq >= 0 && xq < W) {
                            const uint8_t *a = labt + 3 * t, *b = labt + 3 * ((long)yy * W + xq);
                            double e = sqrt((double)(a[0] - b[0]) * (a[0] - b[0]) + (double)(a[1] - b[1]) * (a[1] - b[1]) +
                                            (double)(a[2] - b[2]) * (a[2] - b[2]));
                            wt = pw * exp(-e / gamma_s);
                        }
                        double wgt = wr * wt;
                        sw += wgt;
                        sc += wgt * cost[d + (long)D * ((long)wrap1(yy, H) * W + wrap1(xr, W))];
                    }
                }
                out[d + (long)D * p] = sc / sw;
            }
        }
}

/* The same FP64 aggregation as orc64_aw_l2r over an FP64 cost volume, with
 * every pixel's weights computed once (the sums in the same tap order). */
int orc64_aw_l2r_pre(const uint8_t *labr, const uint8_t *labt, const double *cost, double *out,
                     int H, int W, int D, int rad, double gamma_s, double gamma_p) {
    int edge = 2 * rad + 1;
    long E = (long)edge * edge, np = (long)H * W;
    double *wr = (double *)malloc(sizeof(double) * np * E), *wt = (double *)malloc(sizeof(double) * np * E);
    if (!wr || !wt) { free(wr); free(wt); return -1; }
    for (int pass = 0; pass < 2; pass++) {
        const uint8_t *lab = pass ? labt : labr;
        double *w = pass ? wt : wr;
        ORC_PAR
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                long p = (long)y * W + x, k = 0;
                for (int dy = -rad; dy <= rad; dy++)
                    for (int dx = -rad; dx <= rad; dx++, k++) {
                        int yy = y + dy, xx = x + dx;
                        double v = 0;
                        if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
                            const uint8_t *a = lab + 3 * p, *b = lab + 3 * ((long)yy * W + xx);
                            double e = sqrt((double)(a[0] - b[0]) * (a[0] - b[0]) + (double)(a[1] - b[1]) * (a[1] - b[1]) +
                                            (double)(a[2] - b[2]) * (a[2] - b[2]));
                            v = exp(-sqrt((double)(dy * dy + dx * dx)) / gamma_p) * exp(-e / gamma_s);
                        }
                        w[p * E + k] = v;
                    }
            }
    }
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            for (int d = 0; d < D; d++) {
                long t = (long)y * W + tar_col(x, d, W, ORC_L2R);
                double sw = 0, sc = 0;
                long k = 0;
                for (int dy = -rad; dy <= rad; dy++)
                    for (int dx = -rad; dx <= rad; dx++, k++) {
                        double wgt = wr[p * E + k] * wt[t * E + k];
                        sw += wgt;
                        sc += wgt * cost[d + (long)D * ((long)wrap1(y + dy, H) * W + wrap1(x + dx, W))];
                    }
                out[d + (long)D * p] = sc / sw;
            }
        }
    free(wr);
    free(wt);
    return 0;
}

void orc64_ncc(const uint8_t *ref, const uint8_t *tar, double *cost, int D, int H, int W, int hrad, int wrad) {
    int area = (2 * hrad + 1) * (2 * wrad + 1);
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            long p = (long)y * W + x;
            double mr = 0;
            for (int dy = -hrad; dy <= hrad; dy++)
                for (int dx = -wrad; dx <= wrad; dx++)
                    mr += ref[(long)wrap1(y + dy, H) * W + wrap1(x + dx, W)];
            mr /= area;
            for (int d = 0; d < D; d++) {
                double mt = 0, nom = 0, den = 0;
                for (int dy = -hrad; dy <= hrad; dy++)
                    for (int dx = -wrad; dx <= wrad; dx++)
                        mt += tar[(long)wrap1(y + dy, H) * W + wrap1(x + dx - d, W)];
                mt /= area;
                for (int dy = -hrad; dy <= hrad; dy++)
                    for (int dx = -wrad; dx <= wrad; dx++) {
                        double rv = ref[(long)wrap1(y + dy, H) * W + wrap1(x + dx, W)] - mr;
                        double tv = tar[(long)wrap1(y + dy, H) * W + wrap1(x + dx - d, W)] - mt;
                        nom += rv * tv;
                        den += rv * rv * tv * tv;
                    }
                den = sqrt(den);
                cost[d + (long)D * p] = (den != 0) ? nom / den : NAN;
            }
        }
}

void orc64_convolve(const uint8_t *img, double *out, const float *mask, int H, int W, int hrad, int wrad) {
    int mw = 2 * wrad + 1;
    ORC_PAR
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            double acc = 0;
            for (int dy = -hrad; dy <= hrad; dy++)
                for (int dx = -wrad; dx <= wrad; dx++)
                    acc += (double)img[(long)wrap1(y + dy, H) * W + wrap1(x + dx, W)] * (double)mask[(dy + hrad) * mw + (dx + wrad)];
            acc = fabs(acc);
            out[(long)y * W + x] = acc > 255 ? 255 : acc;
        }
}

/* ------------------------------------------------------------------------- */
/* Pipeline: seq/Main.cpp:180-257 for one view.                               */

static void flip_rows(const uint8_t *src, uint8_t *dst, int H, int W, int ch) {
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int c = 0; c < ch; c++)
                dst[((long)y * W + x) * ch + c] = src[((long)y * W + (W - 1 - x)) * ch + c];
}

/* one matching cost into `cost` (seq/Main.cpp:180-231); trunc_ad selects the
 * truncated colour AD (cross-based aggregation with AD as the first cost). */
static int one_cost(const orc_params *p, int which, int trunc_ad, int H, int W, const uint8_t *rg,
                    const uint8_t *tg, const uint8_t *rc, const uint8_t *tc, float *cost) {
    long np = (long)H * W;
    int D = p->D;
    switch (which) {
    case 1:
        orc_ad_color(rc, tc, cost, D, H, W, ORC_L2R, trunc_ad, p->ad_trunc, 0);
        return 0;
    case 2: {
        uint8_t *a = (uint8_t *)malloc(np), *b = (uint8_t *)malloc(np);
        if (!a || !b) { free(a); free(b); return -1; }
        orc_rank(rg, a, p->rank_rad, H, W);
        orc_rank(tg, b, p->rank_rad, H, W);
        orc_ad_gray(a, b, cost, D, H, W, ORC_L2R);
        free(a); free(b);
        return 0;
    }
    case 3: {
        long nb = (long)(2 * p->census_hrad + 1) * (2 * p->census_wrad + 1);
        uint8_t *a = (uint8_t *)malloc(np * nb), *b = (uint8_t *)malloc(np * nb);
        if (!a || !b) { free(a); free(b); return -1; }
        orc_census(rg, a, p->census_hrad, p->census_wrad, H, W);
        orc_census(tg, b, p->census_hrad, p->census_wrad, H, W);
        orc_hamming(a, b, cost, p->census_hrad, p->census_wrad, H, W, D);
        free(a); free(b);
        return 0;
    }
    case 4: {
        float *a = (float *)malloc(np * sizeof(float)), *b = (float *)malloc(np * sizeof(float));
        if (!a || !b) { free(a); free(b); return -1; }
        orc_convolve(rg, a, orc_log5x5, H, W, 2, 2);
        orc_convolve(tg, b, orc_log5x5, H, W, 2, 2);
        orc_ad_float(a, b, cost, D, H, W, ORC_L2R);
        free(a); free(b);
        return 0;
    }
    case 5:
        /* NCC leaves den==0 cells unwritten; start from 0 like a fresh buffer */
        memset(cost, 0, sizeof(float) * np * D);
        orc_ncc(rg, tg, cost, D, H, W, p->ncc_hrad, p->ncc_wrad);
        return 0;
    }
    return -1;
}

/* The matching cost of one view (seq/Main.cpp:180-234): cost1 (truncated colour
 * AD when cost1 is AD in a cross-based run), and cost2 combined into it. */
int orc_view_cost(const orc_params *p, int H, int W, const uint8_t *rg, const uint8_t *tg, const uint8_t *rc,
                  const uint8_t *tc, float *cost) {
    if (one_cost(p, p->cost1, p->aggr == 3, H, W, rg, tg, rc, tc, cost)) return -1;
    if (!p->cost2) return 0;
    long ne = (long)H * W * p->D;
    float *c2 = (float *)malloc(ne * sizeof(float));
    if (!c2 || one_cost(p, p->cost2, 0, H, W, rg, tg, rc, tc, c2)) {
        free(c2);
        return -1;
    }
    orc_combine(cost, c2, p->lambda1, p->lambda2, H, W, p->D);
    free(c2);
    return 0;
}

/* ra / ta: the images the cross arms are found on (the colour images, or
 * their median-filtered copies) */
static int one_view(const orc_params *p, int H, int W, const uint8_t *rg, const uint8_t *tg,
                    const uint8_t *rc, const uint8_t *tc, const uint8_t *rl, const uint8_t *tl,
                    const uint8_t *ra, const uint8_t *ta, uint8_t *disp, float *cost_out) {
    long np = (long)H * W, ne = np * p->D;
    int D = p->D, rc_ = -1;
    float *c1 = (float *)malloc(ne * sizeof(float)), *c3 = NULL;
    if (!c1) return -1;
    if (orc_view_cost(p, H, W, rg, tg, rc, tc, c1)) goto out;
    float *fin = c1;
    if (p->aggr == 1) {
        if (p->box_inplace) orc_box_inplace(c1, H, W, D, p->box_rad);
        else {
            c3 = (float *)malloc(ne * sizeof(float));
            if (!c3) goto out;
            orc_box(c1, c3, H, W, D, p->box_rad);
            fin = c3;
        }
    } else if (p->aggr == 2) {
        int edge = 2 * p->aw_rad + 1;
        long area = (long)edge * edge;
        float *pw = (float *)malloc(area * sizeof(float));
        float *wr = (float *)malloc(np * area * sizeof(float));
        float *wt = (float *)malloc(np * area * sizeof(float));
        c3 = (float *)malloc(ne * sizeof(float));
        if (!pw || !wr || !wt || !c3) { free(pw); free(wr); free(wt); goto out; }
        orc_prox_weight(pw, p->aw_gamma_p, p->aw_rad);
        orc_compute_weights(wr, pw, rl, p->aw_gamma_s, H, W, p->aw_rad);
        orc_compute_weights(wt, pw, tl, p->aw_gamma_s, H, W, p->aw_rad);
        orc_aw_l2r(wr, wt, c1, c3, H, W, D, p->aw_rad);
        free(pw); free(wr); free(wt);
        fin = c3;
    } else if (p->aggr == 3) {
        int *hr = (int *)malloc(np * 2 * sizeof(int)), *ht = (int *)malloc(np * 2 * sizeof(int));
        int *vr = (int *)malloc(np * 2 * sizeof(int)), *vt = (int *)malloc(np * 2 * sizeof(int));
        c3 = (float *)malloc(ne * sizeof(float));
        if (!hr || !ht || !vr || !vt || !c3) { free(hr); free(ht); free(vr); free(vt); goto out; }
        orc_find_cross(ra, hr, vr, H, W, p->cross_L, p->cross_tau);
        orc_find_cross(ta, ht, vt, H, W, p->cross_L, p->cross_tau);
        orc_prefix_h(c1, H, W, D);
        orc_cross_aggr(c1, c3, hr, ht, vr, vt, H, W, D);
        free(hr); free(ht); free(vr); free(vt);
        fin = c3;
    }
    orc_wta(fin, disp, H, W, D, p->cost1 == 5 && p->cost2 == 0);
    if (cost_out) memcpy(cost_out, fin, ne * sizeof(float));
    rc_ = 0;
out:
    free(c1); free(c3);
    return rc_;
}

int orc_pipeline(const orc_params *p, int H, int W,
                 const uint8_t *lgray, const uint8_t *rgray,
                 const uint8_t *lrgb, const uint8_t *rrgb,
                 const uint8_t *llab, const uint8_t *rlab,
                 uint8_t *disp_left, uint8_t *disp_right, uint8_t *mask, float *cost_out) {
    if (!p || H <= 0 || W <= 0 || p->D <= 0 || p->D > 256 || p->D > W) return -1;
    if (p->median_ksize && (p->median_ksize < 3 || p->median_ksize > 15 || !(p->median_ksize & 1))) return -1;
    long np = (long)H * W;
    /* the OpenCL driver's cross path: arms from median-filtered colour images */
    uint8_t *med = NULL;
    const uint8_t *la = lrgb, *ra = rrgb;
    if (p->median_ksize && p->aggr == 3) {
        med = (uint8_t *)malloc(np * 12);
        if (!med) return -1;
        orc_median(lrgb, med, H, W, 3, p->median_ksize);
        orc_median(rrgb, med + 3 * np, H, W, 3, p->median_ksize);
        la = med;
        ra = med + 3 * np;
    }
    if (one_view(p, H, W, lgray, rgray, lrgb, rrgb, llab, rlab, la, ra, disp_left, cost_out)) {
        free(med);
        return -1;
    }
    if (!p->right_view) {
        free(med);
        return 0;
    }
    uint8_t *buf = (uint8_t *)malloc(np * 14 + np);
    if (!buf) {
        free(med);
        return -1;
    }
    uint8_t *fg_l = buf, *fg_r = fg_l + np, *fc_l = fg_r + np, *fc_r = fc_l + 3 * np;
    uint8_t *fl_l = fc_r + 3 * np, *fl_r = fl_l + 3 * np, *fd = fl_r + 3 * np;
    uint8_t *fa_l = fc_l, *fa_r = fc_r;
    if (med) {
        fa_l = med + 6 * np;
        fa_r = med + 9 * np;
        flip_rows(la, fa_l, H, W, 3);
        flip_rows(ra, fa_r, H, W, 3);
    }
    flip_rows(lgray, fg_l, H, W, 1);
    flip_rows(rgray, fg_r, H, W, 1);
    flip_rows(lrgb, fc_l, H, W, 3);
    flip_rows(rrgb, fc_r, H, W, 3);
    if (llab && rlab) {
        flip_rows(llab, fl_l, H, W, 3);
        flip_rows(rlab, fl_r, H, W, 3);
    }
    int rc = one_view(p, H, W, fg_r, fg_l, fc_r, fc_l, fl_r, fl_l, fa_r, fa_l, fd, NULL);
    if (rc == 0) {
        flip_rows(fd, disp_right, H, W, 1);
        orc_cross_check(disp_left, disp_right, mask, H, W);
    }
    free(buf);
    free(med);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Synthetic inputs for the CPU legs that must not load the product library   */
/* (the timed reference arm).  The same generator as the library's            */
/* rts_synth_pair / rts_gray_to_rgb / rts_rgb_to_lab: xoshiro256** seeded by   */
/* splitmix64, 3x3 box-smoothed uniform texture, rectangles and slanted planes */
/* of constant disparity, Box-Muller noise, rounding half away from zero, and */
/* the CIE L*a*b* formulas (sRGB, D65) with 8-bit scaling.  The reference has */
/* no generator; tests/test_oracle_synth.py checks the two bit for bit.       */

typedef struct { uint64_t s[4]; } orc_rng;

static uint64_t rng_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static void rng_seed(orc_rng *r, uint64_t seed) {
    uint64_t z = seed;
    for (int i = 0; i < 4; i++) {
        z += 0x9e3779b97f4a7c15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
        r->s[i] = x ^ (x >> 31);
    }
}

static uint64_t rng_next(orc_rng *r) {
    uint64_t *s = r->s;
    const uint64_t res = rng_rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rng_rotl(s[3], 45);
    return res;
}

static int rng_below(orc_rng *r, int n) { return (int)((rng_next(r) >> 11) % (uint64_t)n); }
static double rng_unit(orc_rng *r) { return ((rng_next(r) >> 11) + 1) * (1.0 / 9007199254740992.0); }
static double rng_gauss(orc_rng *r) {
    const double u1 = rng_unit(r), u2 = rng_unit(r);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}
static int round_half_away(double v) { return v < 0 ? -(int)floor(-v + 0.5) : (int)floor(v + 0.5); }
static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

int orc_synth_pair(uint64_t seed, int W, int H, int max_disp, int n_rects, int n_planes, float sigma, int bg_disp,
                   uint8_t *left, uint8_t *right, uint8_t *gt) {
    if (W <= 0 || H <= 0 || max_disp <= 0 || max_disp > 256 || !left || !right || n_rects < 0 || n_planes < 0)
        return -1;
    orc_rng rng;
    rng_seed(&rng, seed);
    const long np = (long)W * H;
    uint8_t *raw = (uint8_t *)malloc(np), *d = (uint8_t *)malloc(np);
    if (!raw || !d) { free(raw); free(d); return -1; }
    for (long i = 0; i < np; i++) raw[i] = (uint8_t)(rng_next(&rng) >> 56);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int s = 0;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++)
                    s += raw[(long)clampi(y + dy, 0, H - 1) * W + clampi(x + dx, 0, W - 1)];
            left[(long)y * W + x] = (uint8_t)((s + 4) / 9);
        }
    memset(d, clampi(bg_disp, 0, max_disp - 1), np);
    for (int i = 0; i < n_rects; i++) {
        const int rw = 1 + rng_below(&rng, W / 3 > 1 ? W / 3 : 1), rh = 1 + rng_below(&rng, H / 3 > 1 ? H / 3 : 1);
        const int x0 = rng_below(&rng, W), y0 = rng_below(&rng, H), dv = rng_below(&rng, max_disp);
        for (int y = y0; y < y0 + rh && y < H; y++)
            for (int x = x0; x < x0 + rw && x < W; x++) d[(long)y * W + x] = (uint8_t)dv;
    }
    for (int i = 0; i < n_planes; i++) {
        const int rw = 1 + rng_below(&rng, W / 2 > 1 ? W / 2 : 1), rh = 1 + rng_below(&rng, H / 2 > 1 ? H / 2 : 1);
        const int x0 = rng_below(&rng, W), y0 = rng_below(&rng, H);
        const double a = rng_below(&rng, max_disp);
        const double b = (rng_unit(&rng) - 0.5) * 2.0 * (double)max_disp / (double)W;
        const double c = (rng_unit(&rng) - 0.5) * 2.0 * (double)max_disp / (double)H;
        for (int y = y0; y < y0 + rh && y < H; y++)
            for (int x = x0; x < x0 + rw && x < W; x++)
                d[(long)y * W + x] = (uint8_t)clampi(round_half_away(a + b * (x - x0) + c * (y - y0)), 0, max_disp - 1);
    }
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const int dv = d[(long)y * W + x];
            const double v = left[(long)y * W + clampi(x + dv, 0, W - 1)] + (sigma > 0 ? sigma * rng_gauss(&rng) : 0.0);
            right[(long)y * W + x] = (uint8_t)clampi(round_half_away(v), 0, 255);
        }
    if (gt) memcpy(gt, d, np);
    free(raw);
    free(d);
    return 0;
}

void orc_gray_to_rgb(const uint8_t *gray, uint8_t *rgb, int W, int H) {
    const long np = (long)W * H;
    for (long i = 0; i < np; i++) rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = gray[i];
}

static double srgb_to_linear(double c) { return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4); }
static double lab_f(double t) { return t > 216.0 / 24389.0 ? cbrt(t) : (24389.0 / 27.0 * t + 16.0) / 116.0; }

void orc_rgb_to_lab(const uint8_t *rgb, uint8_t *lab, int W, int H) {
    const long np = (long)W * H;
    for (long i = 0; i < np; i++) {
        const double r = srgb_to_linear(rgb[3 * i] / 255.0), g = srgb_to_linear(rgb[3 * i + 1] / 255.0),
                     b = srgb_to_linear(rgb[3 * i + 2] / 255.0);
        const double X = (0.4124564 * r + 0.3575761 * g + 0.1804375 * b) / 0.95047;
        const double Y = 0.2126729 * r + 0.7151522 * g + 0.0721750 * b;
        const double Z = (0.0193339 * r + 0.1191920 * g + 0.9503041 * b) / 1.08883;
        const double fx = lab_f(X), fy = lab_f(Y), fz = lab_f(Z);
        const double L = 116.0 * fy - 16.0, A = 500.0 * (fx - fy), B = 200.0 * (fy - fz);
        lab[3 * i] = (uint8_t)clampi(round_half_away(L * 255.0 / 100.0), 0, 255);
        lab[3 * i + 1] = (uint8_t)clampi(round_half_away(A + 128.0), 0, 255);
        lab[3 * i + 2] = (uint8_t)clampi(round_half_away(B + 128.0), 0, 255);
    }
}
