"""Batched form (rts_batch_run: one launch per stage for all pairs, CUDA graph
replay, autotuned tiles) and the serving loop (rts_server_*): every pair's
result is the same as its single-pair pipeline run -- alone and in the mix --
and the single-pair run is pinned to the oracle elsewhere."""
import time

import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu

MIX = [(160, 120, 32), (96, 64, 64), (200, 90, 16), (128, 128, 128), (64, 48, 32), (250, 60, 64)]
# disparity ranges above 128: eight 32-disparity chunks per lane, a partial last one
WIDE = [(300, 40, 256), (96, 64, 64), (260, 33, 200), (180, 20, 130)]


def make_pairs(seed0, mix=MIX):
    import rtstereo_gb300 as R
    out = []
    for i, (W, H, D) in enumerate(mix):
        L, Rr, _ = R.synth_pair(seed0 + i, W, H, D, 4, 1, 2.0, min(4, D - 1))
        out.append((L, Rr, D))
    return out


def single(ctx, L, Rr, D, prec):
    import rtstereo_gb300 as R
    return ctx.pipeline(R.params(disp_range=D, precision=prec), L, Rr)[:3]


@pytest.mark.parametrize("mix", ["mix", "wide"])
@pytest.mark.parametrize("prec", [0, 1])
def test_batch_matches_single_runs(ctx, oracle_mod, prec, mix):
    torch = pytest.importorskip("torch")
    import rtstereo_gb300 as R
    s = torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)
    try:
        for rnd in range(2):  # the second round replays the captured graph with new data
            data = make_pairs(1000 * rnd + 7, MIX if mix == "mix" else WIDE)
            dev, pairs, params, outs, bufs = [], [], [], [], []
            for L, Rr, D in data:
                H, W = L.shape
                dl, dr = torch.from_numpy(L).cuda(), torch.from_numpy(Rr).cuda()
                o = [torch.zeros((H, W), dtype=torch.uint8, device="cuda") for _ in range(3)]
                dev.append((dl, dr))
                bufs.append(o)
                pairs.append(R.Pair(W, H, dl.data_ptr(), dr.data_ptr(), None, None, None, None))
                params.append(R.params(disp_range=D, precision=prec))
                outs.append(R.Out(o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), None))
            s.wait_stream(torch.cuda.current_stream())
            ctx.batch_run(pairs, params, outs)
            s.synchronize()
            for (L, Rr, D), o in zip(data, bufs):
                want = single(ctx, L, Rr, D, prec)
                for g, w in zip(o, want):
                    assert bits_equal(g.cpu().numpy(), w)
    finally:
        ctx.set_stream(None)
    # and the plain single-pair run itself equals the oracle for one of them
    if prec == 0 and mix == "mix":
        L, Rr, D = make_pairs(7)[0]
        O = oracle_mod
        rgb = lambda a: np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))
        o = O.pipeline(O.params(D=D), L, Rr, rgb(L), rgb(Rr))
        g = single(ctx, L, Rr, D, 0)
        assert all(bits_equal(a, b) for a, b in zip(g, o[:3]))


@pytest.mark.parametrize("priority_pixels,pinned", [(0, False), (128 * 128, False), (128 * 128, True)])
def test_server_same_alone_and_in_the_mix(ctx, priority_pixels, pinned):
    """With priority_pixels the larger pairs of the mix run alone on high-priority
    streams while the smaller ones are batched; with pinned result buffers the
    device writes them directly; results do not change."""
    import rtstereo_gb300 as R
    torch = pytest.importorskip("torch") if pinned else None
    srv = R.Server(ctx, hbm_budget=1 << 30, max_inflight=8, max_batch=3, precision=R.PREC_F16,
                   priority_pixels=priority_pixels)
    try:
        data = make_pairs(55) * 3
        tickets = []
        for L, Rr, D in data:
            outs = None
            if pinned:
                outs = tuple(torch.full(L.shape, 77, dtype=torch.uint8).pin_memory().numpy() for _ in range(3))
            tickets.append(srv.submit(R.params(disp_range=D, precision=R.PREC_F16), L, Rr, outs=outs))
            srv.progress()
        stats = [srv.wait(t) for t, _ in tickets]
        for (L, Rr, D), (t, outs) in zip(data, tickets):
            want = single(ctx, L, Rr, D, R.PREC_F16)
            for g, w in zip(outs, want):
                assert bits_equal(g, w)
        assert all(s[0] <= s[1] <= s[2] for s in stats)
    finally:
        srv.close()


def test_server_admission_and_cancel(ctx):
    import rtstereo_gb300 as R
    # a small budget: a large request is refused outright, small ones queue for memory
    srv = R.Server(ctx, hbm_budget=24 << 20, max_inflight=2, max_batch=1, precision=R.PREC_F16)
    try:
        L, Rr, _ = R.synth_pair(3, 1024, 768, 128, 4, 0, 2.0, 4)
        with pytest.raises(R.RtsError) as e:
            srv.submit(R.params(disp_range=128, precision=R.PREC_F16), L, Rr)
        assert e.value.status == 6  # RTS_ERR_BUSY: larger than the server's HBM budget
        data = make_pairs(9)[:5]
        tickets = [srv.submit(R.params(disp_range=D, precision=R.PREC_F16), a, b)[0] for a, b, D in data]
        assert srv.cancel(tickets[-1]) == 0
        for t in tickets[:-1]:
            srv.wait(t)
        with pytest.raises(R.RtsError) as e:
            srv.wait(tickets[-1])
        assert e.value.status == 7  # RTS_ERR_CANCELLED
    finally:
        srv.close()


def test_server_large_pair_overtakes_held_small_one(ctx):
    """priority_pixels: while a large pair runs, a small one waits, and a large pair
    submitted after it starts first; every result is still the single-pair run's."""
    import rtstereo_gb300 as R
    srv = R.Server(ctx, hbm_budget=4 << 30, max_inflight=8, max_batch=2, precision=R.PREC_F16,
                   priority_pixels=1920 * 1080)
    try:
        big = [R.synth_pair(0xB0 + i, 1920, 1080, 128, 8, 1, 2.0, 4)[:2] for i in range(2)]
        small = R.synth_pair(0xB5, 320, 240, 32, 4, 0, 2.0, 4)[:2]
        order = [(big[0], 128), (small, 32), (big[1], 128)]

        def run():
            tickets = []
            for (L, Rr), D in order:
                tickets.append(srv.submit(R.params(disp_range=D, precision=R.PREC_F16), L, Rr))
                srv.progress()
            return tickets, [srv.wait(t) for t, _ in tickets]

        run()  # warm: the server's pinned staging for these sizes, the kernels
        tickets, stats = run()
        # (submit, start, done) in ms: the first large pair runs for milliseconds, so
        # the small pair is held and the second large pair is launched before it
        assert stats[2][1] <= stats[1][1]
        assert stats[1][1] >= stats[0][0]
        for ((L, Rr), D), (t, outs) in zip(order, tickets):
            for g, w in zip(outs, single(ctx, L, Rr, D, R.PREC_F16)):
                assert bits_equal(g, w)
    finally:
        srv.close()


def test_server_cancel_while_held(ctx):
    """A small request cancelled while held behind a running large one leaves the
    queue cleanly; the large requests around it finish with their single-pair
    results."""
    import rtstereo_gb300 as R
    srv = R.Server(ctx, hbm_budget=4 << 30, max_inflight=8, max_batch=2, precision=R.PREC_F16,
                   priority_pixels=1920 * 1080)
    try:
        big = [R.synth_pair(0xC0 + i, 1920, 1080, 64, 8, 1, 2.0, 4)[:2] for i in range(2)]
        small = [R.synth_pair(0xC5 + i, 320, 240, 32, 4, 0, 2.0, 4)[:2] for i in range(2)]
        p = lambda D: R.params(disp_range=D, precision=R.PREC_F16)
        # warm: pinned staging for these sizes (pinning pages takes milliseconds,
        # long enough for the first large pair to finish before the small one arrives)
        for t, _ in [srv.submit(p(64), *big[0]), srv.submit(p(32), *small[0]), srv.submit(p(32), *small[1]),
                     srv.submit(p(64), *big[1])]:
            srv.wait(t)
        ta, oa = srv.submit(p(64), *big[0])
        srv.progress()
        ts1, _ = srv.submit(p(32), *small[0])
        ts2, os2 = srv.submit(p(32), *small[1])
        assert srv.cancel(ts1) == 0
        tb, ob = srv.submit(p(64), *big[1])
        srv.progress()
        srv.wait(ta)
        srv.wait(tb)
        srv.wait(ts2)
        with pytest.raises(R.RtsError) as e:
            srv.wait(ts1)
        assert e.value.status == 7  # RTS_ERR_CANCELLED
        for (L, Rr), D, outs in ((big[0], 64, oa), (big[1], 64, ob), (small[1], 32, os2)):
            for g, w in zip(outs, single(ctx, L, Rr, D, R.PREC_F16)):
                assert bits_equal(g, w)
        # every request was collected or cancelled: the server holds none
        assert srv.tracked() == 0
        # a request cancelled while it runs is dropped when its batch leaves the device
        tc, _ = srv.submit(p(64), *big[0])
        srv.progress()
        assert srv.cancel(tc) == 0
        t_end = time.time() + 10.0
        while srv.tracked() and time.time() < t_end:
            srv.progress()
        assert srv.tracked() == 0
        with pytest.raises(R.RtsError) as e:
            srv.wait(tc)
        assert e.value.status == 7  # RTS_ERR_CANCELLED, from the record of cancelled tickets
    finally:
        srv.close()
