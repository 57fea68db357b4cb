"""rts_WTA_noalloc: winner-takes-all for callers that cannot allocate device
memory (a host that fixes its device memory at start-up, or a frame loop that
must not stall on cudaMalloc's device-wide synchronisation).  Its scratch is a
static device array inside the library, so this test checks that two calls in a
row, through the C ABI on device buffers, give exactly what rts_WTA gives --
the second call must not see the first call's leftovers."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def carry_heavy_cost(seed, H, W, D):
    rng = np.random.default_rng(seed)
    cost = rng.integers(0, 4, (H, W, D)).astype(np.float32)
    cost[:, :, 0] = 0  # many pixels keep the previous winner (seq/WTA.cpp:12)
    cost[H // 3:H // 2] = 1
    cost[H // 3:H // 2, :, 0] = 0  # whole rows without a winner of their own
    return cost


def test_noalloc_matches_wta_on_two_calls():
    torch = pytest.importorskip("torch")
    import rtstereo_gb300 as R
    lib = R.lib()
    with R.Context(0) as ctx:
        stream = torch.cuda.Stream()
        for seed, (H, W, D) in ((1, (120, 97, 16)), (2, (200, 160, 64))):
            cost = carry_heavy_cost(seed, H, W, D)
            want = ctx.WTA(cost)  # the existing entry point
            dcost = torch.from_numpy(cost).cuda()
            out = torch.full((H, W), 77, dtype=torch.uint8, device="cuda")
            stream.wait_stream(torch.cuda.current_stream())
            st = lib.rts_WTA_noalloc(C.c_void_p(dcost.data_ptr()), C.c_void_p(out.data_ptr()), H, W, D,
                                     C.c_void_p(stream.cuda_stream))
            assert st == 0
            stream.synchronize()
            assert np.array_equal(out.cpu().numpy(), want)


def test_noalloc_rejects_sizes_beyond_its_array():
    import rtstereo_gb300 as R
    lib = R.lib()
    # 2048 x 2048 pixels is above the 2,097,152-pixel limit; rejected before any device work
    assert lib.rts_WTA_noalloc(C.c_void_p(16), C.c_void_p(16), 2048, 2048, 16, None) == 1
    assert lib.rts_WTA_noalloc(C.c_void_p(16), C.c_void_p(16), 9000, 4, 2, None) == 1
