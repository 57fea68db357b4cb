// Replays the row-ring schedule of the vertical cross-aggregation kernel
// (k_vert_views) on the host with the kernel's own constants
// (rts_vert_ring.h) and checks, for every arm length the fused path takes
// (0..23) and every strip start, that
//   * every row a step reads has been ingested by that step's barrier,
//   * no row a step reads has been overwritten by a later ingest,
//   * the tick a fast warp may ingest during that step (the next step's) writes
//     no slot a slow warp still reads,
//   * the depth is a multiple of 8 and the first slot index is below it.
// Prints the largest distance (newest row written - oldest row read) + 1 per
// arm length and exits 1 on the first violation.
#include <stdio.h>

#include <algorithm>

#include "rts_vert_ring.h"

using rts::vert_depth;
using rts::vert_first_ticks;

static int fail(const char *what, int L, int y0, int s, int r) {
    printf("FAIL %s: L=%d y0=%d step=%d row=%d depth=%d\n", what, L, y0, s, r, vert_depth(L));
    return 1;
}

int main() {
    for (int L = 0; L <= 23; L++) {
        const int DEP = vert_depth(L);
        if (DEP % 8 != 0 || DEP < 2 * L + 23) return fail("depth", L, 0, 0, 0);
        int worst = 0;
        // strips start at y0 (a multiple of the strip height, or 0); what matters is
        // y0 - ra = min(y0, L) and where the image ends (rb)
        for (int y0 = 0; y0 <= L + 24; y0++)
            for (int tail = 0; tail <= L + 9; tail++) {
                const int nrows = 40;               // rows of the strip
                const int y1 = y0 + nrows, H = y1 + tail;
                const int ra = std::max(0, y0 - L), rb = std::min(H, y1 + L);
                const int T0 = vert_first_ticks(y0, ra, L);
                if (y0 - ra >= DEP) return fail("first slot", L, y0, 0, y0);
                const int nsteps = (y1 - y0 + 7) >> 3;
                auto slot = [&](int r) { return (r - ra) % DEP; };
                for (int s = 0; s < nsteps; s++) {
                    const int ingested = std::min(rb, ra + 8 * (T0 + s)) - 1;  // newest row after step s's ingest
                    const int lo_read = std::max(ra, y0 + 8 * s - L);
                    for (int w = 0; w < 8; w++) {
                        const int y = y0 + 8 * s + w;
                        if (y >= y1) break;
                        for (int r = std::max(0, y - L); r <= std::min(H - 1, y + L); r++) {
                            if (r < ra || r >= rb) return fail("row outside the ring's range", L, y0, s, r);
                            if (r > ingested) return fail("row read before its ingest", L, y0, s, r);
                            if (ingested - r >= DEP) return fail("row overwritten before its read", L, y0, s, r);
                            // the next tick, ingested by a warp that runs ahead
                            for (int w2 = 0; w2 < 8; w2++) {
                                const int r2 = ra + 8 * (T0 + s) + w2;
                                if (r2 >= rb) break;
                                if (slot(r2) == slot(r)) return fail("slot written while read", L, y0, s, r);
                            }
                        }
                    }
                    const int newest = std::min(rb - 1, ra + 8 * (T0 + s) + 7);
                    worst = std::max(worst, newest - lo_read + 1);
                }
            }
        printf("L=%d depth=%d needed=%d\n", L, DEP, worst);
        if (worst > DEP) return fail("depth below the needed rows", L, -1, -1, -1);
    }
    printf("ok\n");
    return 0;
}
