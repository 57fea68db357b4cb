// rts_common.cuh -- device helpers shared by the kernels of rtstereo_gb300.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "rts_internal.h"

namespace rts {

// Single wrap of an index that is at most one period outside [0, n): the
// reference's border rule (e.g. seq/CensusTransform.cpp:21-22).
__device__ __forceinline__ int wrap1(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Target column of disparity d: dir > 0 => x-d (+W if negative, L2R,
// seq/PixelBasedCost.cpp:19-20); dir < 0 => x+d (-W if >= W, R2L, :32-33).
__device__ __forceinline__ int tar_col(int x, int d, int W, int dir) {
    if (dir > 0) {
        int t = x - d;
        return t < 0 ? t + W : t;
    }
    int t = x + d;
    return t >= W ? t - W : t;
}

// Dynamic shared memory one block may opt into on sm_100-class GPUs (227 KB);
// kernels whose tile sizes are compile-time constants assert against it.
constexpr size_t kSmemOptin = 227 * 1024;

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

// WTA order key of cost v at disparity d (seq/WTA.cpp:10-39): the least {key, d}
// over d is the reference's winner -- the first strict minimum (maximum with
// argmax) in increasing d.  Keys order like the floats, -0 == +0; a NaN never wins
// (the largest key), and a NaN at d = 0 blocks every other d (the smallest key,
// which no number takes).
__device__ __forceinline__ uint32_t wta_key(float v, int d, int argmax) {
    if (v != v) return d == 0 ? 0u : 0xffffffffu;
    uint32_t u = __float_as_uint(__fadd_rn(v, 0.0f));  // -0 -> +0
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return argmax ? ~u : u;
}
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }

// Packed cross arms of one pixel: left | right<<8 | top<<16 | bottom<<24.
__device__ __forceinline__ int arm_l(uint32_t a) { return (int)(a & 0xff); }
__device__ __forceinline__ int arm_r(uint32_t a) { return (int)((a >> 8) & 0xff); }
__device__ __forceinline__ int arm_t(uint32_t a) { return (int)((a >> 16) & 0xff); }
__device__ __forceinline__ int arm_b(uint32_t a) { return (int)(a >> 24); }

// One term of CombineCost (seq/CombineCost.cpp:21-22): 1 - exp(-v/lambda).
// Integer-valued costs in range take it from a table computed on the host with
// the C library's expf (the reference's arithmetic, so bit-identical); other
// values use the device expf (within a few ulp).
__device__ __forceinline__ float combine_term(float v, const float *__restrict__ lut, float lambda) {
    if (v >= 0.f && v < (float)kCombineLut && v == truncf(v)) return lut[(int)v];
    return __fsub_rn(1.0f, expf(__fdiv_rn(-v, lambda)));
}

// packed pairs of floats for the f32x2 instructions
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float half2_of(unsigned long long v, int hi) {
    float lo_, hi_;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo_), "=f"(hi_) : "l"(v));
    return hi ? hi_ : lo_;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

}  // namespace rts
