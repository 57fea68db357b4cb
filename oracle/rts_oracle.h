/*
 * rts_oracle.h -- CPU oracle for the rtstereo per-frame stereo pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * sequential implementation (rtstereo seq/ sources).  Only tests/, the smoke check
 * in __graft_entry__.py and the CPU-baseline leg of bench.py may load it, and
 * only as the checker or the timed CPU baseline -- never as the product path.
 *
 * Every function states the reference file:line range it follows.  Layouts are
 * the reference's:  gray u8 [H][W]; RGB/Lab u8 [H][W][3]; cost volume f32
 * [H][W][D] indexed cost[d + D*(x + W*y)]; census bits u8 (0/1) [H][W][N].
 * Float arithmetic is written in the reference's order with float temporaries;
 * the file must be compiled with -ffp-contract=off so that no multiply-add is
 * fused (the reference, built with g++ -O2 on x86-64, fuses none).
 */
#ifndef RTS_ORACLE_H
#define RTS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* direction of the target lookup: +1 => target x-d (L2R), -1 => target x+d (R2L) */
enum { ORC_L2R = 1, ORC_R2L = -1 };

void orc_ad_gray(const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int dir);
void orc_ad_float(const float *ref, const float *tar, float *cost, int D, int H, int W, int dir);
void orc_ad_color(const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W,
                  int dir, int use_trunc, float trunc, int norm);
void orc_census(const uint8_t *img, uint8_t *bits, int hrad, int wrad, int H, int W);
void orc_hamming(const uint8_t *bref, const uint8_t *btar, float *cost, int hrad, int wrad,
                 int H, int W, int D);
void orc_rank(const uint8_t *img, uint8_t *out, int rad, int H, int W);
void orc_convolve(const uint8_t *img, float *out, const float *mask, int H, int W, int hrad, int wrad);
void orc_ncc(const uint8_t *ref, const uint8_t *tar, float *cost, int D, int H, int W, int hrad, int wrad);
void orc_combine(float *c1, const float *c2, float lambda1, float lambda2, int H, int W, int D);
void orc_box_inplace(float *cost, int H, int W, int D, int rad);
void orc_box(const float *cost, float *out, int H, int W, int D, int rad);
void orc_find_cross(const uint8_t *rgb, int *horz, int *vert, int H, int W, int arm_len, int tau);
/* OpenCV medianBlur as opencl/Main.cpp:342-343 uses it: per channel, the middle
 * value of the k x k window, border pixels replicated (k odd). */
void orc_median(const uint8_t *img, uint8_t *out, int H, int W, int ch, int k);
void orc_prefix_h(float *cost, int H, int W, int D);
void orc_cross_aggr(const float *pre, float *out, const int *hr, const int *ht, const int *vr,
                    const int *vt, int H, int W, int D);
void orc_prox_weight(float *pw, float gamma_p, int rad);
void orc_compute_weights(float *w, const float *pw, const uint8_t *lab, float gamma_s, int H, int W, int rad);
void orc_aw_l2r(const float *wref, const float *wtar, const float *cost, float *out, int H, int W, int D, int rad);
/* the same two steps for rows y0 .. y0+nrows-1 only (weights and output hold those rows) */
void orc_compute_weights_rows(float *w, const float *pw, const uint8_t *lab, float gamma_s, int H, int W, int rad,
                              int y0, int nrows);
void orc_aw_l2r_rows(const float *wref, const float *wtar, const float *cost, float *out, int H, int W, int D,
                     int rad, int y0, int nrows);
void orc_aw_r2l(const float *wref, const float *wtar, float *cost, int H, int W, int D, int rad);
/* out-of-place forms of the two in-place functions (the GPU contract) */
void orc_aw_r2l_oop(const float *wref, const float *wtar, const float *cost, float *out, int H, int W, int D, int rad);
void orc_wta(const float *cost, uint8_t *win, int H, int W, int D, int argmax);
void orc_cross_check(const uint8_t *dref, const uint8_t *dtar, uint8_t *mask, int H, int W);
void orc_disp_refinement(uint8_t *disp, const int *horz, const int *vert, int H, int W, int D);
void orc_disp_refinement_oop(const uint8_t *disp, uint8_t *out, const int *horz, const int *vert, int H, int W, int D);

/* FP64 restatements (same loops, double arithmetic) for error reports. */
void orc64_combine(const float *c1, const float *c2, double lambda1, double lambda2, long n, double *out);
void orc64_aw_l2r(const uint8_t *labr, const uint8_t *labt, const float *cost, double *out,
                  int H, int W, int D, int rad, double gamma_s, double gamma_p);
int orc64_aw_l2r_pre(const uint8_t *labr, const uint8_t *labt, const double *cost, double *out,
                     int H, int W, int D, int rad, double gamma_s, double gamma_p);
void orc64_ncc(const uint8_t *ref, const uint8_t *tar, double *cost, int D, int H, int W, int hrad, int wrad);
void orc64_convolve(const uint8_t *img, double *out, const float *mask, int H, int W, int hrad, int wrad);

/* Whole-pipeline restatement of seq/Main.cpp:180-257 (left view) plus the right
 * view as flip(L2R(flip(R), flip(L))) and the cross check. */
typedef struct {
    int cost1, cost2;     /* 1 AD, 2 rank, 3 census, 4 LoG, 5 NCC; cost2 = 0 => single cost */
    int aggr;             /* 0 none, 1 box, 2 adaptive weight, 3 cross-based */
    float lambda1, lambda2;
    int D;
    int census_hrad, census_wrad;
    int rank_rad;
    int ncc_hrad, ncc_wrad;
    int box_rad;
    int aw_rad;
    float aw_gamma_s, aw_gamma_p;
    int cross_L, cross_tau;
    float ad_trunc;
    int right_view;       /* 1: also compute the right view and the cross-check mask */
    int box_inplace;      /* 1: the literal in-place box of the reference */
    int median_ksize;     /* 0, or odd: cross arms from median-filtered colour images
                             (opencl/Main.cpp:342-343); costs from the unfiltered ones */
} orc_params;

/* Returns 0 on success, -1 on allocation failure or bad parameters.  cost_out
 * (optional, may be NULL) receives the left view's final cost volume. */
int orc_pipeline(const orc_params *p, int H, int W,
                 const uint8_t *lgray, const uint8_t *rgray,
                 const uint8_t *lrgb, const uint8_t *rrgb,
                 const uint8_t *llab, const uint8_t *rlab,
                 uint8_t *disp_left, uint8_t *disp_right, uint8_t *mask, float *cost_out);

/* One view's matching cost volume (cost1, and cost2 combined into it), as the
 * pipeline makes it.  Returns 0, or -1 on allocation failure. */
int orc_view_cost(const orc_params *p, int H, int W, const uint8_t *rg, const uint8_t *tg, const uint8_t *rc,
                  const uint8_t *tc, float *cost);

/* Host threads for the row loops (n <= 0: all processors); 1 when built without OpenMP. */
void orc_set_threads(int n);
int orc_threads(void);

/* Seeded random-dot pairs and colour conversions, the same generator as the
 * library's rts_synth_pair / rts_gray_to_rgb / rts_rgb_to_lab (the CPU legs
 * that must not load the library make their inputs with these). */
int orc_synth_pair(uint64_t seed, int W, int H, int max_disp, int n_rects, int n_planes, float sigma, int bg_disp,
                   uint8_t *left, uint8_t *right, uint8_t *gt);
void orc_gray_to_rgb(const uint8_t *gray, uint8_t *rgb, int W, int H);
void orc_rgb_to_lab(const uint8_t *rgb, uint8_t *lab, int W, int H);

/* the 5x5 LoG mask of the reference driver (seq/Main.cpp:113-117) */
extern const float orc_log5x5[25];

#ifdef __cplusplus
}
#endif
#endif
