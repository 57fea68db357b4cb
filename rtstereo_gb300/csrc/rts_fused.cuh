// rts_fused.cuh -- device helpers shared by the fused pipeline kernels
// (k_pipe.cu, k_batch.cu): costs from per-pixel records, storage conversions,
// order-preserving float keys for warp arg-min.
#pragma once

#include <cuda_fp16.h>

#include "rts_common.cuh"

namespace rts {

// ---------------------------------------------------------------------------
// cost of one (ref pixel, target pixel) pair from records

struct CostCfg {
    int k1, k2;        // RTS_COST_AD / RTS_COST_CENSUS; k2 may be RTS_COST_NONE
    int trunc1;        // truncated AD for the first cost (cross-based aggregation)
    float trunc;
    const float *lut1, *lut2;
    float l1, l2;
    int int_path;      // 1: both costs are integers < kCombineLut (integral truncation)
    int itrunc;        // integral truncation, or a large value when not truncating
};

// Integer value of one cost from records: SAD of the packed RGB bytes (the
// fourth byte is zero) or the census Hamming distance.
__device__ __forceinline__ int rec_icost(int kind, const uint4 &a, const uint4 &b, int itrunc) {
    if (kind == RTS_COST_CENSUS) return __popc(a.x ^ b.x) + __popc(a.y ^ b.y);
    return imin((int)__vsadu4(a.z, b.z), itrunc);
}

__device__ __forceinline__ float rec_cost(int kind, const uint4 &a, const uint4 &b, int use_trunc, float trunc) {
    if (kind == RTS_COST_CENSUS) {
        const uint64_t ca = ((uint64_t)a.y << 32) | a.x, cb = ((uint64_t)b.y << 32) | b.x;
        return (float)__popcll(ca ^ cb);  // seq/CensusTransform.cpp:52-60
    }
    // seq/PixelBasedCost.cpp:86-91 / :106-112 with normOrNot = 0
    const int sad = abs((int)(a.z & 0xff) - (int)(b.z & 0xff)) + abs((int)((a.z >> 8) & 0xff) - (int)((b.z >> 8) & 0xff)) +
                    abs((int)((a.z >> 16) & 0xff) - (int)((b.z >> 16) & 0xff));
    float v = (float)sad;
    if (use_trunc) v = (v > trunc) ? trunc : v;
    return v;
}

__device__ __forceinline__ float pair_cost(const uint4 &a, const uint4 &b, const CostCfg &c) {
    const float v1 = rec_cost(c.k1, a, b, c.trunc1, c.trunc);
    if (c.k2 == RTS_COST_NONE) return v1;
    const float v2 = rec_cost(c.k2, a, b, 0, 0.f);
    return __fadd_rn(combine_term(v1, c.lut1, c.l1), combine_term(v2, c.lut2, c.l2));  // seq/CombineCost.cpp:23
}

template <typename T> __device__ __forceinline__ T to_store(float v);
template <> __device__ __forceinline__ float to_store<float>(float v) { return v; }
template <> __device__ __forceinline__ __half to_store<__half>(float v) { return __float2half_rn(v); }
// integer costs: v is an exact non-negative integer below 2^16
template <> __device__ __forceinline__ uint16_t to_store<uint16_t>(float v) { return (uint16_t)__float2uint_rn(v); }
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }

__device__ __forceinline__ uint32_t order_key(float v) {
    const uint32_t u = __float_as_uint(__fadd_rn(v, 0.0f));  // -0 -> +0
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

}  // namespace rts
