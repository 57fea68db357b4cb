// rts_tma.h -- TMA (cp.async.bulk.tensor) support: a cost volume [H][W][D] as a
// 3-D tensor map, and the bounded mbarrier wait the staging kernels use.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rts {

// The volume [H][W][D] of elem-byte values as a 3-D tensor map (d, x, y) with box
// (bd, bw, bh), zeros past the edges.  False where a TMA rule fails (rows of D
// values a multiple of 16 bytes, a 16-byte aligned base, boxes of at most 256 per
// dimension) or the driver has no encoder; callers then stage by cp.async.
inline bool volume_tensor_map(CUtensorMap *m, const void *vol, int H, int W, int D, int elem, int bd, int bw,
                              int bh) {
    // looked up once (a function-local static: thread-safe initialisation)
    static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        const bool ok = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                                         &q) == cudaSuccess &&
                        q == cudaDriverEntryPointSuccess;
        return ok ? (PFN_cuTensorMapEncodeTiled_v12000)fn : (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    if (!encode || ((size_t)D * elem) % 16 != 0 || ((uintptr_t)vol & 15) != 0) return false;
    if (bd > 256 || bw > 256 || bh > 256 || ((size_t)bd * elem) % 16 != 0) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)D, (cuuint64_t)W, (cuuint64_t)H};
    const cuuint64_t strides[2] = {(cuuint64_t)D * elem, (cuuint64_t)W * D * elem};
    const cuuint32_t box[3] = {(cuuint32_t)bd, (cuuint32_t)bw, (cuuint32_t)bh};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType t = elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    return encode(m, t, 3, const_cast<void *>(vol), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

#ifdef __CUDACC__
constexpr int kTmaSpin = 1 << 22;  // polls of an mbarrier before a wait gives up

// Waits for the phase of parity `parity` of the mbarrier at shared address bar;
// false after kTmaSpin polls.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < kTmaSpin; it++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: a 3-D tile copy of `bytes` bytes at (c0, c1, c2) into shared dst,
// completing on bar.  The proxy fence orders earlier generic accesses of the
// destination (the block's previous use of the buffer) before the copy.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint32_t bar, uint32_t bytes) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}
#endif

}  // namespace rts
