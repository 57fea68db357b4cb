"""Host-side helpers of bench.py on CPU: the numpy FP64 adaptive-weight
reference the FP16 bench line reports against (checked against the oracle's
FP64 restatement), and the roofline arithmetic of the JSON line."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_numpy_f64_adaptive_weights_match_oracle(oracle_mod):
    import bench
    import rtstereo_gb300 as R
    O = oracle_mod
    H, W, D, rad = 30, 48, 12, 16
    L, Rr, _ = R.synth_pair(9, W, H, D, 3, 0, 2.0, 4)
    Lc, Rc = R.gray_to_rgb(L), R.gray_to_rgb(Rr)
    Ll, Rl = R.rgb_to_lab(Lc), R.rgb_to_lab(Rc)
    rows = [0, 7, 29]
    got = bench.f64_aw_rows(L, Rr, Lc, Rc, Ll, Rl, D, rad, 7.0, 36.0, 10.0, 10.0, rows, 4, 3)
    c1 = O.ad_color(Lc, Rc, D)
    c2 = O.hamming(O.census(L), O.census(Rr), D)
    want = O.f64_aw_l2r_pre(Ll, Rl, O.f64_combine(c1, c2, 10.0, 10.0), rad, 7.0, 36.0)[rows]
    assert np.abs(got - want).max() < 1e-12


def test_roofline_fields():
    import bench
    import rtstereo_gb300 as R
    peaks = {"hbm_gbs": 6000.0, "sm_max_mhz": 2000.0}
    # adaptive weights: FP32-pipe bound, 4 ops per tap per entry
    p = R.params(aggr=2, disp_range=64)
    r = bench.roofline({"aw_wta": (2, 8.0)}, "aw_640x480_d64", 640, 480, 64, 2, peaks, "measured", p)
    assert r["bound"] == "fp32" and r["kernel"] == "k_aw_wta_pipe"
    assert r["ms_per_launch"] == pytest.approx(4.0)
    assert r["ops_per_launch"] == pytest.approx(4 * 33 * 33 * 640 * 480 * 64)
    assert r["peak"] == pytest.approx(152 * 128 * 2000e6 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["binding_unit"]["unit"].startswith("L1") and 0 < r["binding_unit"]["busy_ncu"] <= 1
    # the SM count is the device's (passed in), the FP16 form counts 3 operations a tap
    r16 = bench.roofline({"aw_wta": (2, 8.0)}, "aw_640x480_d64", 640, 480, 64, 2, peaks, "measured",
                         R.params(aggr=2, disp_range=64, precision=R.PREC_F16), sms=160)
    assert r16["peak"] == pytest.approx(160 * 128 * 2000e6 / 1e12) and "160 SMs" in r16["peak_source"]
    assert r16["ops_per_launch"] == pytest.approx(3 * 33 * 33 * 640 * 480 * 64)
    # the FP16 form aggregates once: the left-view scope around it is not a kernel
    r16 = bench.roofline({"left_view": (1, 3.3), "aw_wta": (1, 3.2), "right_view": (1, 0.1)}, "aw_640x480_d64",
                         640, 480, 64, 2, peaks, "measured", R.params(aggr=2, disp_range=64, precision=R.PREC_F16))
    assert r16["kernel"] == "k_aw_wta_pipe" and r16["ms_per_launch"] == pytest.approx(3.2)
    # box: FP32-pipe bound, (2r+1)^2 adds per entry, one launch per view
    p = R.params(aggr=1, disp_range=128, box_rad=4)
    r = bench.roofline({"box_wta": (2, 2.0), "left_view": (1, 1.5)}, "box_1920x1080_d128", 1920, 1080, 128, 1,
                       peaks, "measured", p)
    assert r["bound"] == "fp32" and r["kernel"] == "k_box_best_dp" and r["ms_per_launch"] == pytest.approx(1.0)
    assert r["ops_per_launch"] == pytest.approx(81 * 1920 * 1080 * 128) and r["traffic"] == pytest.approx(1.1375e9)
    # NCC 7x7 volume: FP32-pipe bound, 5 operations per tap per entry
    p = R.params(aggr=1, disp_range=128, box_rad=4, cost1=5, cost2=0, ncc_hrad=3, ncc_wrad=3)
    r = bench.roofline({"cost": (2, 6.0), "box_wta": (2, 2.0)}, "ncc_box_1920x1080_d128", 1920, 1080, 128, 1,
                       peaks, "measured", p)
    assert r["bound"] == "fp32" and r["kernel"] == "k_ncc_tiled" and r["ms_per_launch"] == pytest.approx(3.0)
    assert r["ops_per_launch"] == pytest.approx(5 * 49 * 1920 * 1080 * 128)
    # cross-based: HBM stage model, 2 views x 2 crossings x S bytes per entry
    p = R.params(disp_range=128)
    stages = {"cross_hseg": (1, 1.0), "cross_vert_wta": (1, 2.0)}
    r = bench.roofline(stages, "cross_1920x1080_d128", 1920, 1080, 128, 3, peaks, "measured", p, ms_pair=3.5)
    E = 1920 * 1080 * 128
    assert r["kernel"] == "cross_vert_wta" and r["bytes_per_launch"] == 2 * 2 * 4 * E
    assert r["traffic"] == pytest.approx(4.16 * 2 * E)
    assert r["pipeline"]["bytes_per_pair"] == 2 * (4 * 4 * E) + 2 * (8 * 1920 * 1080) + 3 * 1920 * 1080
    # integer costs keep 2-byte segments, with their own ncu traffic figure
    p = R.params(disp_range=128, cost1=3, cost2=0)
    r = bench.roofline(stages, "census_cross_1920x1080_d128", 1920, 1080, 128, 3, peaks, "measured", p)
    assert r["bytes_per_launch"] == 2 * 2 * 2 * E and r["traffic"] == pytest.approx(2.13 * 2 * E)


def test_reference_arm_line():
    """bench.py --impl reference on a small strip: one JSON line with the
    reference-arm keys; the sample runs the reference's own code where it is
    built (kind "reference"), else the oracle port."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                          "--cpu-rows", "4", "--workload", "cross_384x288_d16"], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    import oracle
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "MDE/s"
    assert line["cpu_baseline"]["kind"] == ("reference" if oracle.have_reference() else "port")
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    # the same config object as the GPU arm prints for this workload
    import bench as B
    assert line["config"] == B.workload_config("cross_384x288_d16", "f32", 1)


def test_reference_arm_does_not_load_the_library():
    """The CPU reference arm makes its inputs with the oracle's copy of the
    generator: neither it nor its workers map the product library."""
    import subprocess
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--cpu-rows', '4', '--workload', 'cross_384x288_d16']\n"
            "if __name__ == '__main__':\n"
            "    import bench; bench.main()\n"
            "    print('MAPS', 'librtstereo_gb300' in open('/proc/self/maps').read())\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "MAPS False" in out.stdout


def test_latency_target_record():
    import bench
    by = {"1920x1080": {"n": 12, "p99": 4.9, "from_arrival_p99": 5.2}, "320x240": {"n": 3, "p99": 1.0,
                                                                             "from_arrival_p99": 1.1}}
    r = bench.latency_target(by, "1920x1080", 5.0)
    assert r == {"size": "1920x1080", "n": 12, "target_ms": 5.0, "p99_ms": 4.9, "from_arrival_p99_ms": 5.2,
                 "met": True}
    assert bench.latency_target(by, "1280x720", 5.0) is None
    by["1920x1080"]["p99"] = 5.0
    assert bench.latency_target(by, "1920x1080", 5.0)["met"] is False


def test_c2_box_record_fields():
    """The default line's box sub-record from two measured runs (a stand-in for the
    GPU measurement): the FP16 ratio, the agreement of both views and the mask."""
    import bench
    outs = [np.full((4, 6), 7, np.uint8), np.full((4, 6), 5, np.uint8), np.ones((4, 6), np.uint8)]

    class FakeBench:
        def measure(self, name, precision):
            assert name == "box_1920x1080_d128"
            ms = 2.34 if precision == "f32" else 1.30
            o16 = [a.copy() for a in outs]
            if precision == "f16":
                o16[1][0, 0] = 6  # one right-view disparity differs
            return {"ms": ms, "value": 1920 * 1080 * 128 / 1e6 / (ms / 1e3), "e2e": {"ms_per_step": ms + 0.1},
                    "stages_ms_per_step": {"box_wta": ms / 2}, "roofline": {"kernel": "k_box_best_dp", "frac": 0.77},
                    "clocks": {"sm_mhz": 2070.0}, "out": o16}

    r = bench.c2_box_record(FakeBench())
    assert r["workload"] == "box_1920x1080_d128" and r["ms_per_pair"] == pytest.approx(2.34)
    assert r["dominant_kernel"]["kernel"] == "k_box_best_dp"
    assert r["f16"]["ratio_to_plain"] == pytest.approx(2.34 / 1.30)
    assert r["f16"]["agreement"] == {"disp_left": 1.0, "disp_right": pytest.approx(23 / 24), "mask": 1.0}
