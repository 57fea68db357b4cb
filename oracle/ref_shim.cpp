// ref_shim.cpp -- extern "C" entry points over the reference's own seq/*.cpp.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's seq/ sources (read where they lie, never copied) into
// oracle/_ref/libseqref.so, which the tests use to pin the C restatement in
// rts_oracle.c and to make the golden fixtures.  The prototypes below restate
// the reference's declarations (seq/*.h) so that its C++ symbols link; the
// reference headers are not included because they define min/max/square macros.

// seq/PixelBasedCost.h:6-13 (the R2L colour variants are defined as pixelBasedR2L_Color,
// seq/PixelBasedCost.cpp:116,138)
void pixelBasedL2R(unsigned char *, unsigned char *, float *, const int, const int, const int);
void pixelBasedR2L(unsigned char *, unsigned char *, float *, const int, const int, const int);
void pixelBasedCostL2R_Float(float *, float *, float *, const int, const int, const int);
void pixelBasedCostR2L_Float(float *, float *, float *, const int, const int, const int);
void pixelBasedCostL2R_Color(unsigned char *, unsigned char *, float *, const int, const int, const int, int);
void pixelBasedCostL2R_Color(unsigned char *, unsigned char *, float *, const int, const int, const int, float, int);
void pixelBasedR2L_Color(unsigned char *, unsigned char *, float *, const int, const int, const int, int);
void pixelBasedR2L_Color(unsigned char *, unsigned char *, float *, const int, const int, const int, float, int);
// seq/CensusTransform.h:1-2
void calcCensusTrans(unsigned char *, bool *, const int, const int, const int, const int);
void calcHammingDist(bool *, bool *, float *, const int, const int, int, int, int);
// seq/RankFilter.h:1, seq/ConvolveImage.h:1, seq/NCCDisparity.h:3, seq/CombineCost.h:3
void calculateRankFilt(unsigned char *, unsigned char *, const int, const int, const int);
void convolveImage(unsigned char *, float *, float *, const int, const int, const int, const int);
void calcNCCDispL2R(unsigned char *, unsigned char *, float *, const int, const int, const int, const int, const int);
void combineCost(float *, float *, float, float, int, int, int);
// seq/ConstBlockAggregation.h:1
void boxAggregate(float *, const int, const int, const int, const int);
// seq/CrossBasedAggregation.h:14-19
void findCross(unsigned char *, int *, int *, int, int);
void aggregate_cost_horizontal(float *, int, int, int);
void cross_stereo_aggregation(float *, float *, int *, int *, int *, int *, int, int, int);
void disp_refinement(unsigned char *, int *, int *, int, int, int);
// seq/AdaptiveWeightAggreagtion.h:4-10
void calcProxWeight(float *, float, int);
void computeWeights(float *, float *, unsigned char *, const float, const int, const int, const int);
void calcAWCostL2R(float *, float *, float *, float *, const int, const int, const int, const int);
void calcAWCostR2L(float *, float *, float *, const int, const int, const int, const int);
// seq/WTA.h:1-2, seq/CrossCheck.h:1
void WTA(float *, unsigned char *, const int, const int, const int);
void WTA_NCC(float *, unsigned char *, const int, const int, const int);
void cross_check(unsigned char *, unsigned char *, unsigned char *, const int, const int);

extern "C" {
typedef unsigned char u8;

void ref_pixelBasedL2R(u8 *r, u8 *t, float *c, int D, int H, int W) { pixelBasedL2R(r, t, c, D, H, W); }
void ref_pixelBasedR2L(u8 *r, u8 *t, float *c, int D, int H, int W) { pixelBasedR2L(r, t, c, D, H, W); }
void ref_pixelBasedCostL2R_Float(float *r, float *t, float *c, int D, int H, int W) { pixelBasedCostL2R_Float(r, t, c, D, H, W); }
void ref_pixelBasedCostR2L_Float(float *r, float *t, float *c, int D, int H, int W) { pixelBasedCostR2L_Float(r, t, c, D, H, W); }
void ref_pixelBasedCostL2R_Color(u8 *r, u8 *t, float *c, int D, int H, int W, int norm) { pixelBasedCostL2R_Color(r, t, c, D, H, W, norm); }
void ref_pixelBasedCostL2R_Color_trunc(u8 *r, u8 *t, float *c, int D, int H, int W, float tr, int norm) { pixelBasedCostL2R_Color(r, t, c, D, H, W, tr, norm); }
void ref_pixelBasedR2L_Color(u8 *r, u8 *t, float *c, int D, int H, int W, int norm) { pixelBasedR2L_Color(r, t, c, D, H, W, norm); }
void ref_pixelBasedR2L_Color_trunc(u8 *r, u8 *t, float *c, int D, int H, int W, float tr, int norm) { pixelBasedR2L_Color(r, t, c, D, H, W, tr, norm); }
void ref_calcCensusTrans(u8 *img, u8 *bits, int hr, int wr, int H, int W) { calcCensusTrans(img, (bool *)bits, hr, wr, H, W); }
void ref_calcHammingDist(u8 *a, u8 *b, float *c, int hr, int wr, int H, int W, int D) { calcHammingDist((bool *)a, (bool *)b, c, hr, wr, H, W, D); }
void ref_calculateRankFilt(u8 *img, u8 *out, int m, int H, int W) { calculateRankFilt(img, out, m, H, W); }
void ref_convolveImage(u8 *img, float *out, float *mask, int H, int W, int hr, int wr) { convolveImage(img, out, mask, H, W, hr, wr); }
void ref_calcNCCDispL2R(u8 *r, u8 *t, float *c, int D, int H, int W, int hr, int wr) { calcNCCDispL2R(r, t, c, D, H, W, hr, wr); }
void ref_combineCost(float *a, float *b, float l1, float l2, int H, int W, int D) { combineCost(a, b, l1, l2, H, W, D); }
void ref_boxAggregate(float *c, int H, int W, int D, int r) { boxAggregate(c, H, W, D, r); }
void ref_findCross(u8 *rgb, int *h, int *v, int H, int W) { findCross(rgb, h, v, H, W); }
void ref_aggregate_cost_horizontal(float *c, int H, int W, int D) { aggregate_cost_horizontal(c, H, W, D); }
void ref_cross_stereo_aggregation(float *c, float *o, int *hr, int *ht, int *vr, int *vt, int H, int W, int D) {
    cross_stereo_aggregation(c, o, hr, ht, vr, vt, H, W, D);
}
void ref_disp_refinement(u8 *d, int *h, int *v, int H, int W, int D) { disp_refinement(d, h, v, H, W, D); }
void ref_calcProxWeight(float *pw, float gp, int r) { calcProxWeight(pw, gp, r); }
void ref_computeWeights(float *w, float *pw, u8 *lab, float gs, int H, int W, int r) { computeWeights(w, pw, lab, gs, H, W, r); }
void ref_calcAWCostL2R(float *wr, float *wt, float *c, float *o, int H, int W, int D, int r) { calcAWCostL2R(wr, wt, c, o, H, W, D, r); }
void ref_calcAWCostR2L(float *wr, float *wt, float *c, int H, int W, int D, int r) { calcAWCostR2L(wr, wt, c, H, W, D, r); }
void ref_WTA(float *c, u8 *w, int H, int W, int D) { WTA(c, w, H, W, D); }
void ref_WTA_NCC(float *c, u8 *w, int H, int W, int D) { WTA_NCC(c, w, H, W, D); }
void ref_cross_check(u8 *a, u8 *b, u8 *m, int H, int W) { cross_check(a, b, m, H, W); }
}
