"""Median pre-filter of the cross arms (the OpenCL driver's medianBlur before
findCross, opencl/Main.cpp:342-343) on the GPU: the module entry point
rts_medianFilt and the pipeline option median_ksize on every cross-based path
(fused view kernels, precomputed-volume views, the composed modules, the
batched form and the serving loop), bit-exact against the oracle."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def colour_pair(seed, W, H, D):
    import rtstereo_gb300 as R
    L, Rr, _ = R.synth_pair(seed, W, H, D, 4, 1, 4.0, min(4, D - 1))
    rng = np.random.default_rng(seed)
    noise = rng.integers(-40, 41, (H, W), dtype=np.int16)
    g = lambda a: np.clip(a.astype(np.int16) + noise, 0, 255).astype(np.uint8)
    Lc = np.ascontiguousarray(np.stack([L, g(L), L // 2], -1))
    Rc = np.ascontiguousarray(np.stack([Rr, g(Rr), Rr // 2], -1))
    return L, Rr, Lc, Rc


def rgb(a):
    return np.ascontiguousarray(np.repeat(a[:, :, None], 3, axis=2))


@pytest.mark.parametrize("H,W", [(1, 1), (2, 3), (9, 40), (67, 129), (130, 33)])
@pytest.mark.parametrize("ch", [1, 3])
@pytest.mark.parametrize("k", [3, 5, 7, 15])
def test_median_filter_matches_oracle(ctx, oracle_mod, H, W, ch, k):
    rng = np.random.default_rng(H * 7919 + W * 31 + k + ch)
    img = rng.integers(0, 256, (H, W) if ch == 1 else (H, W, 3), dtype=np.uint8)
    assert bits_equal(ctx.medianFilt(img, k), oracle_mod.median(img, k))


def test_median_filter_device_in_place(ctx, oracle_mod):
    torch = pytest.importorskip("torch")
    import rtstereo_gb300 as R
    H, W = 70, 90
    img = np.random.default_rng(3).integers(0, 256, (H, W, 3), dtype=np.uint8)
    d = torch.from_numpy(img).cuda()
    torch.cuda.synchronize()
    ctx.call("medianFilt", R.DEVICE, d, H, W, 3, 3)
    ctx.synchronize()
    assert bits_equal(d.cpu().numpy(), oracle_mod.median(img, 3))


# (cost1, cost2, colour, right_view, k, want_cost): fused record costs, gray-only
# records, a precomputed volume (LoG), the composed modules (cost volume asked for)
CASES = [(1, 3, True, 1, 3, False), (1, 3, False, 1, 3, False), (1, 0, True, 0, 5, False),
         (4, 0, True, 1, 3, False), (1, 3, True, 1, 3, True), (3, 0, False, 1, 15, False)]


@pytest.mark.parametrize("c1,c2,colour,right,k,want_cost", CASES)
def test_pipeline_median_matches_oracle(ctx, oracle_mod, c1, c2, colour, right, k, want_cost):
    import rtstereo_gb300 as R
    O = oracle_mod
    W, H, D = 150, 70, 32
    L, Rr, Lc, Rc = colour_pair(0x3E0 + c1 * 10 + k, W, H, D)
    if not colour:
        Lc, Rc = rgb(L), rgb(Rr)
    p = R.params(cost1=c1, cost2=c2, disp_range=D, right_view=right, median_ksize=k)
    g = ctx.pipeline(p, L, Rr, Lc if colour else None, Rc if colour else None, want_cost=want_cost)
    o = O.pipeline(O.params(cost1=c1, cost2=c2, D=D, right_view=right, median_ksize=k), L, Rr, Lc, Rc,
                   want_cost=want_cost)
    assert bits_equal(g[0], o[0])
    if right:
        assert bits_equal(g[1], o[1]) and bits_equal(g[2], o[2])
    if want_cost:
        assert bits_equal(g[3], o[3])
    # the option is not a no-op on these inputs
    plain = O.pipeline(O.params(cost1=c1, cost2=c2, D=D, right_view=right), L, Rr, Lc, Rc)
    assert not np.array_equal(plain[0], o[0])


def test_batch_and_server_median_match_oracle(ctx, oracle_mod):
    torch = pytest.importorskip("torch")
    import rtstereo_gb300 as R
    O = oracle_mod
    shapes = [(160, 120, 32), (96, 64, 64), (200, 90, 16)]
    data = [colour_pair(0x5E0 + i, W, H, D) + (D,) for i, (W, H, D) in enumerate(shapes)]
    want = [O.pipeline(O.params(D=D, median_ksize=3), L, Rr, Lc, Rc)[:3] for L, Rr, Lc, Rc, D in data]
    for rnd in range(2):  # the second call replays the captured graph
        keep, pairs, params, outs, bufs = [], [], [], [], []
        for L, Rr, Lc, Rc, D in data:
            H, W = L.shape
            t = [torch.from_numpy(a).cuda() for a in (L, Rr, Lc, Rc)]
            o = [torch.zeros((H, W), dtype=torch.uint8, device="cuda") for _ in range(3)]
            keep.append(t)
            bufs.append(o)
            pairs.append(R.Pair(W, H, *[a.data_ptr() for a in t], None, None))
            params.append(R.params(disp_range=D, median_ksize=3))
            outs.append(R.Out(o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), None))
        torch.cuda.synchronize()
        ctx.batch_run(pairs, params, outs)
        ctx.synchronize()
        for o, w in zip(bufs, want):
            assert all(bits_equal(a.cpu().numpy(), b) for a, b in zip(o, w))
    srv = R.Server(ctx, hbm_budget=1 << 30, max_inflight=4, max_batch=2, precision=R.PREC_F32)
    try:
        tickets = [srv.submit(R.params(disp_range=D, median_ksize=3), L, Rr, Lc, Rc) for L, Rr, Lc, Rc, D in data]
        for t, _ in tickets:
            srv.wait(t)
        for (t, outs), w in zip(tickets, want):
            assert all(bits_equal(a, b) for a, b in zip(outs, w))
    finally:
        srv.close()


def test_median_option_validated(ctx):
    import rtstereo_gb300 as R
    L = np.zeros((16, 32), np.uint8)
    for kw in (dict(median_ksize=4), dict(median_ksize=17), dict(median_ksize=3, aggr=1)):
        with pytest.raises(R.RtsError):
            ctx.pipeline(R.params(disp_range=8, **kw), L, L)
    with pytest.raises(R.RtsError):
        ctx.medianFilt(np.zeros((4, 4), np.uint8), 2)


def test_fp16_server_with_median_and_priority(ctx):
    """FP16 form, median-filtered arms, the priority class and pinned results in
    the serving loop: every result equals the single-pair run of the same form."""
    torch = pytest.importorskip("torch")
    import rtstereo_gb300 as R
    shapes = [(160, 120, 32), (96, 64, 64), (200, 90, 16), (128, 100, 48)]
    data = [colour_pair(0x6E0 + i, W, H, D) + (D,) for i, (W, H, D) in enumerate(shapes)]
    mk = lambda D: R.params(disp_range=D, median_ksize=3, precision=R.PREC_F16)
    want = [ctx.pipeline(mk(D), L, Rr, Lc, Rc)[:3] for L, Rr, Lc, Rc, D in data]
    srv = R.Server(ctx, hbm_budget=1 << 30, max_inflight=4, max_batch=2, precision=R.PREC_F16,
                   priority_pixels=150 * 100)
    try:
        tickets = []
        for L, Rr, Lc, Rc, D in data * 2:
            outs = tuple(torch.zeros(L.shape, dtype=torch.uint8).pin_memory().numpy() for _ in range(3))
            tickets.append(srv.submit(mk(D), L, Rr, Lc, Rc, outs=outs))
        for t, _ in tickets:
            srv.wait(t)
        for (t, outs), w in zip(tickets, want * 2):
            assert all(bits_equal(a, b) for a, b in zip(outs, w))
    finally:
        srv.close()
