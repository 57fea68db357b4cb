// rts_seq_compat.hpp -- the reference's seq/ module API with its exact C++
// signatures (seq/PixelBasedCost.h:6-13, seq/CensusTransform.h:1-2,
// seq/RankFilter.h:1, seq/ConvolveImage.h:1, seq/NCCDisparity.h:3,
// seq/CombineCost.h:3, seq/ConstBlockAggregation.h:1,
// seq/AdaptiveWeightAggreagtion.h:4-10, seq/CrossBasedAggregation.h:14-19,
// seq/WTA.h:1-2, seq/CrossCheck.h:1), implemented over the C ABI in
// rtstereo.h with HOST buffers.  Existing call sites compile unchanged; each
// call copies its inputs to the GPU, runs there, and copies the outputs back.
//
// The functions keep the reference's void return: a non-OK status prints the
// library's message and aborts (the reference has no error path either).
// One library context per thread is created on first use (device 0, or the
// device set with rts_seq_compat_set_device before the first call).
//
// Declared names follow the definitions of seq/ (the R2L colour variants are
// defined as pixelBasedR2L_Color, seq/PixelBasedCost.cpp:116,138).  The
// in-place reference functions boxAggregate, calcAWCostR2L and disp_refinement
// are computed from an unmodified copy of their input (see rtstereo.h).
#pragma once

#include <cstdio>
#include <cstdlib>

#include "rtstereo.h"

namespace rts_compat_detail {
inline int &device() {
    static int d = 0;
    return d;
}
struct Ctx {
    rts_ctx *c = nullptr;
    ~Ctx() {
        if (c) rts_ctx_destroy(c);
    }
};
inline rts_ctx *ctx() {
    thread_local Ctx t;
    if (!t.c) {
        rts_status s = rts_ctx_create(&t.c, device(), 0);
        if (s != RTS_OK) {
            std::fprintf(stderr, "rtstereo: cannot create a context on device %d: %s\n", device(),
                         rts_status_string(s));
            std::abort();
        }
    }
    return t.c;
}
inline void check(rts_status s, const char *fn) {
    if (s != RTS_OK) {
        std::fprintf(stderr, "rtstereo: %s failed: %s (%s)\n", fn, rts_status_string(s), rts_ctx_last_error(ctx()));
        std::abort();
    }
}
}  // namespace rts_compat_detail

inline void rts_seq_compat_set_device(int device) { rts_compat_detail::device() = device; }

#define RTS_COMPAT_CALL(fn, ...) rts_compat_detail::check(fn(rts_compat_detail::ctx(), RTS_HOST, __VA_ARGS__), #fn)

// seq/PixelBasedCost.h:6-13
inline void pixelBasedL2R(unsigned char *ref_image, unsigned char *tar_image, float *cost, const int dispRange,
                          const int rdim, const int cdim) {
    RTS_COMPAT_CALL(rts_pixelBasedL2R, ref_image, tar_image, cost, dispRange, rdim, cdim);
}
inline void pixelBasedR2L(unsigned char *ref_image, unsigned char *tar_image, float *cost, const int dispRange,
                          const int rdim, const int cdim) {
    RTS_COMPAT_CALL(rts_pixelBasedR2L, ref_image, tar_image, cost, dispRange, rdim, cdim);
}
inline void pixelBasedCostL2R_Float(float *ref_image, float *tar_image, float *cost, const int dispRange,
                                    const int rdim, const int cdim) {
    RTS_COMPAT_CALL(rts_pixelBasedCostL2R_Float, ref_image, tar_image, cost, dispRange, rdim, cdim);
}
inline void pixelBasedCostR2L_Float(float *ref_image, float *tar_image, float *cost, const int dispRange,
                                    const int rdim, const int cdim) {
    RTS_COMPAT_CALL(rts_pixelBasedCostR2L_Float, ref_image, tar_image, cost, dispRange, rdim, cdim);
}
inline void pixelBasedCostL2R_Color(unsigned char *ref_image, unsigned char *tar_image, float *cost,
                                    const int dispRange, const int rdim, const int cdim, int normOrNot) {
    RTS_COMPAT_CALL(rts_pixelBasedCostL2R_Color, ref_image, tar_image, cost, dispRange, rdim, cdim, normOrNot);
}
inline void pixelBasedCostL2R_Color(unsigned char *ref_image, unsigned char *tar_image, float *cost,
                                    const int dispRange, const int rdim, const int cdim, float trunc, int normOrNot) {
    RTS_COMPAT_CALL(rts_pixelBasedCostL2R_Color_trunc, ref_image, tar_image, cost, dispRange, rdim, cdim, trunc,
                    normOrNot);
}
inline void pixelBasedR2L_Color(unsigned char *ref_image, unsigned char *tar_image, float *cost, const int dispRange,
                                const int rdim, const int cdim, int normOrNot) {
    RTS_COMPAT_CALL(rts_pixelBasedR2L_Color, ref_image, tar_image, cost, dispRange, rdim, cdim, normOrNot);
}
inline void pixelBasedR2L_Color(unsigned char *ref_image, unsigned char *tar_image, float *cost, const int dispRange,
                                const int rdim, const int cdim, float trunc, int normOrNot) {
    RTS_COMPAT_CALL(rts_pixelBasedR2L_Color_trunc, ref_image, tar_image, cost, dispRange, rdim, cdim, trunc,
                    normOrNot);
}

// seq/CensusTransform.h:1-2
inline void calcCensusTrans(unsigned char *img, bool *censusTrans, const int maskHrad, const int maskWrad,
                            const int rdim, const int cdim) {
    static_assert(sizeof(bool) == 1, "bool must be one byte");
    RTS_COMPAT_CALL(rts_calcCensusTrans, img, reinterpret_cast<uint8_t *>(censusTrans), maskHrad, maskWrad, rdim,
                    cdim);
}
inline void calcHammingDist(bool *censusTrnsRef, bool *censusTrnsTar, float *cost, const int maskHrad,
                            const int maskWrad, int rdim, int cdim, int dispRange) {
    RTS_COMPAT_CALL(rts_calcHammingDist, reinterpret_cast<const uint8_t *>(censusTrnsRef),
                    reinterpret_cast<const uint8_t *>(censusTrnsTar), cost, maskHrad, maskWrad, rdim, cdim,
                    dispRange);
}

// seq/RankFilter.h:1, seq/ConvolveImage.h:1, seq/NCCDisparity.h:3, seq/CombineCost.h:3
inline void calculateRankFilt(unsigned char *img, unsigned char *outImg, const int maskSize, const int rdim,
                              const int cdim) {
    RTS_COMPAT_CALL(rts_calculateRankFilt, img, outImg, maskSize, rdim, cdim);
}
inline void convolveImage(unsigned char *img, float *outIm, float *mask, const int rdim, const int cdim,
                          const int maskHrad, const int maskWrad) {
    RTS_COMPAT_CALL(rts_convolveImage, img, outIm, mask, rdim, cdim, maskHrad, maskWrad);
}
inline void calcNCCDispL2R(unsigned char *ref_image, unsigned char *tar_image, float *cost, const int dispRange,
                           const int rdim, const int cdim, const int maskHrad, const int maskWrad) {
    RTS_COMPAT_CALL(rts_calcNCCDispL2R, ref_image, tar_image, cost, dispRange, rdim, cdim, maskHrad, maskWrad);
}
inline void combineCost(float *cost1, float *cost2, float lambda1, float lambda2, int rdim, int cdim, int dispRange) {
    RTS_COMPAT_CALL(rts_combineCost, cost1, cost2, lambda1, lambda2, rdim, cdim, dispRange);
}

// seq/ConstBlockAggregation.h:1
inline void boxAggregate(float *cost, const int rdim, const int cdim, const int dispRange, const int wndwRad) {
    RTS_COMPAT_CALL(rts_boxAggregate, cost, rdim, cdim, dispRange, wndwRad);
}

// seq/CrossBasedAggregation.h:14-19
inline void findCross(unsigned char *image, int *HorzOffset, int *VertOffset, int rdim, int cdim) {
    RTS_COMPAT_CALL(rts_findCross, image, HorzOffset, VertOffset, rdim, cdim);
}
inline void aggregate_cost_horizontal(float *cost_image, int rdim, int cdim, int dispRange) {
    RTS_COMPAT_CALL(rts_aggregate_cost_horizontal, cost_image, rdim, cdim, dispRange);
}
inline void cross_stereo_aggregation(float *cost_image, float *cost_new_image, int *HorzOffset_ref,
                                     int *HorzOffset_tar, int *VertOffset_ref, int *VertOffset_tar, int rdim,
                                     int cdim, int dispRange) {
    RTS_COMPAT_CALL(rts_cross_stereo_aggregation, cost_image, cost_new_image, HorzOffset_ref, HorzOffset_tar,
                    VertOffset_ref, VertOffset_tar, rdim, cdim, dispRange);
}
inline void disp_refinement(unsigned char *dispIm, int *HorzOffset, int *VertOffset, int rdim, int cdim,
                            int dispRange) {
    RTS_COMPAT_CALL(rts_disp_refinement, dispIm, HorzOffset, VertOffset, rdim, cdim, dispRange);
}

// seq/CrossBasedAggregation.h:12 declares medianFilt(image, maskSize) without
// the image sizes (and never defines it); this overload adds them
inline void medianFilt(unsigned char *image, int maskSize, int rdim, int cdim, int channels = 3) {
    RTS_COMPAT_CALL(rts_medianFilt, image, rdim, cdim, channels, maskSize);
}

// seq/AdaptiveWeightAggreagtion.h:4-10
inline void calcProxWeight(float *proxWeight, float gamma_proximity, int maskRad) {
    RTS_COMPAT_CALL(rts_calcProxWeight, proxWeight, gamma_proximity, maskRad);
}
inline void computeWeights(float *weights, float *proxWeight, unsigned char *LABImage, const float gamma_similarity,
                           const int rdim, const int cdim, const int maskRad) {
    RTS_COMPAT_CALL(rts_computeWeights, weights, proxWeight, LABImage, gamma_similarity, rdim, cdim, maskRad);
}
inline void calcAWCostL2R(float *weightRef, float *weightTar, float *cost, float *newcost, const int rdim,
                          const int cdim, const int dispRange, const int maskRad) {
    RTS_COMPAT_CALL(rts_calcAWCostL2R, weightRef, weightTar, cost, newcost, rdim, cdim, dispRange, maskRad);
}
inline void calcAWCostR2L(float *weightRef, float *weightTar, float *cost, const int rdim, const int cdim,
                          const int dispRange, const int maskRad) {
    RTS_COMPAT_CALL(rts_calcAWCostR2L, weightRef, weightTar, cost, rdim, cdim, dispRange, maskRad);
}

// seq/WTA.h:1-2, seq/CrossCheck.h:1
inline void WTA(float *cost, unsigned char *winners, const int rdim, const int cdim, const int dispRange) {
    RTS_COMPAT_CALL(rts_WTA, cost, winners, rdim, cdim, dispRange);
}
inline void WTA_NCC(float *cost, unsigned char *winners, const int rdim, const int cdim, const int dispRange) {
    RTS_COMPAT_CALL(rts_WTA_NCC, cost, winners, rdim, cdim, dispRange);
}
inline void cross_check(unsigned char *ref_disparity, unsigned char *tar_disparity, unsigned char *cross_check_image,
                        const int rdim, const int cdim) {
    RTS_COMPAT_CALL(rts_cross_check, ref_disparity, tar_disparity, cross_check_image, rdim, cdim);
}

#undef RTS_COMPAT_CALL
