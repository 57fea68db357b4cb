"""include/rts_seq_compat.hpp: a C++ program written against the reference's
seq/ signatures compiles and links against the library unchanged (CPU), and
runs on the GPU to the oracle's results (gpu)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "rtstereo_gb300")

# a call sequence in the reference driver's order (seq/Main.cpp:186-257), AD + census, cross-based
PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "rts_seq_compat.hpp"
int main() {
    const int rdim = 24, cdim = 40, dispRange = 16;
    std::vector<unsigned char> L(rdim * cdim), R(rdim * cdim), Lc(3 * rdim * cdim), Rc(3 * rdim * cdim);
    unsigned s = 12345;
    for (int i = 0; i < rdim * cdim; i++) { s = s * 1103515245u + 12345u; L[i] = (unsigned char)(s >> 24); }
    for (int y = 0; y < rdim; y++) for (int x = 0; x < cdim; x++) R[y * cdim + x] = L[y * cdim + (x + 3) % cdim];
    for (int i = 0; i < rdim * cdim; i++) for (int c = 0; c < 3; c++) { Lc[3 * i + c] = L[i]; Rc[3 * i + c] = R[i]; }
    std::vector<float> c1(rdim * cdim * dispRange), c2(c1.size()), cn(c1.size());
    std::vector<bool> dummy;
    bool *bl = new bool[rdim * cdim * 63], *br = new bool[rdim * cdim * 63];
    std::vector<int> hr(2 * rdim * cdim), vr(hr.size()), ht(hr.size()), vt(hr.size());
    std::vector<unsigned char> disp(rdim * cdim);
    pixelBasedCostL2R_Color(Lc.data(), Rc.data(), c1.data(), dispRange, rdim, cdim, 24.0f, 0);
    calcCensusTrans(L.data(), bl, 4, 3, rdim, cdim);
    calcCensusTrans(R.data(), br, 4, 3, rdim, cdim);
    calcHammingDist(bl, br, c2.data(), 4, 3, rdim, cdim, dispRange);
    combineCost(c1.data(), c2.data(), 10.0f, 10.0f, rdim, cdim, dispRange);
    std::vector<unsigned char> Lm(Lc);  // the median pre-filter overload (result unused)
    medianFilt(Lm.data(), 3, rdim, cdim);
    findCross(Lc.data(), hr.data(), vr.data(), rdim, cdim);
    findCross(Rc.data(), ht.data(), vt.data(), rdim, cdim);
    aggregate_cost_horizontal(c1.data(), rdim, cdim, dispRange);
    cross_stereo_aggregation(c1.data(), cn.data(), hr.data(), ht.data(), vr.data(), vt.data(), rdim, cdim, dispRange);
    WTA(cn.data(), disp.data(), rdim, cdim, dispRange);
    fwrite(disp.data(), 1, disp.size(), stdout);
    delete[] bl; delete[] br;
    return 0;
}
"""


def build_program(tmp_path):
    src = tmp_path / "main.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "main"
    import rtstereo_gb300 as R
    R.lib()
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(ROOT, "include"), "-L", LIBDIR,
                    "-lrtstereo_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], check=True, capture_output=True)
    return exe


def test_compat_header_compiles_and_links(tmp_path):
    assert build_program(tmp_path).exists()


@pytest.mark.gpu
def test_compat_program_matches_oracle(tmp_path, oracle_mod):
    O = oracle_mod
    exe = build_program(tmp_path)
    got = np.frombuffer(subprocess.run([str(exe)], check=True, capture_output=True).stdout, np.uint8).reshape(24, 40)
    rdim, cdim, D = 24, 40, 16
    s = 12345
    L = np.empty(rdim * cdim, np.uint8)
    for i in range(rdim * cdim):
        s = (s * 1103515245 + 12345) & 0xffffffff
        L[i] = s >> 24
    L = L.reshape(rdim, cdim)
    R = np.ascontiguousarray(np.roll(L, -3, axis=1))
    Lc = np.ascontiguousarray(np.repeat(L[:, :, None], 3, axis=2))
    Rc = np.ascontiguousarray(np.repeat(R[:, :, None], 3, axis=2))
    c = O.combine(O.ad_color(Lc, Rc, D, O.L2R, 24.0, 0), O.hamming(O.census(L), O.census(R), D), 10.0, 10.0)
    hl, vl = O.find_cross(Lc)
    ht, vt = O.find_cross(Rc)
    want = O.wta(O.cross_aggr(O.prefix_h(c), hl, ht, vl, vt))
    assert np.array_equal(got, want)
