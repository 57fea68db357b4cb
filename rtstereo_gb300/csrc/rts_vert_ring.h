// rts_vert_ring.h -- the row ring of the vertical cross-aggregation kernel
// (k_vert_views, k_batch.cu): its depth and the ticks ingested before the
// first step.  Plain constexpr arithmetic, shared by the kernel and by the CPU
// test that checks it (tests/test_vert_ring.py compiles this header into a
// small host program).
//
// A block of 8 warps walks one column from row y0; the ring holds rows from
// ra = max(0, y0 - L).  Rows enter 8 at a time ("ticks"): in tick i warp w
// writes row ra + 8 i + w into slot (8 i + w) mod depth.  Step s (one barrier
// each) first ingests tick T0 - 1 + s, then warp w reads rows
// y0 + 8 s + w - L .. y0 + 8 s + w + L.  With one barrier per step a fast
// warp may ingest tick T0 + s (the next step's) while a slow warp still reads
// step s: the newest row then written and the oldest row still read must not
// share a slot.
#pragma once

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace rts {

// Ticks ingested before step 0 reads: every row up to y0 + 7 + L is in the ring.
__host__ __device__ constexpr int vert_first_ticks(int y0, int ra, int L) { return (y0 + 8 + L - ra + 7) >> 3; }

// Ring depth in rows for arm length L.  The newest row a fast warp writes
// during step s is ra + 8 (T0 + s) + 7 and the oldest row a slow warp reads
// is y0 + 8 s - L; with T0 = vert_first_ticks they are at most 2L + 22 rows
// apart (y0 - ra a multiple of 8, e.g. a strip at the image top).  The ring
// holds 2L + 23 rows or more, in whole ticks: a multiple of 8 (so also even,
// and two-row blocks of the walk never straddle the wrap).
__host__ __device__ constexpr int vert_depth(int L) { return 8 * ((2 * L + 23 + 7) / 8); }

}  // namespace rts
