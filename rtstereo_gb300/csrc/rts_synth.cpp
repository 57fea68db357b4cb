// rts_synth.cpp -- seeded synthetic random-dot stereo pairs and colour helpers
// (host code).  The generator is this project's own: xoshiro256** seeded by
// splitmix64, Gaussian noise by Box-Muller, integer rounding half away from
// zero, so the same seed gives the same pair on every host.
#include <math.h>
#include <string.h>

#include <vector>

#include "../../include/rtstereo.h"

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (auto &v : s) {
            z += 0x9e3779b97f4a7c15ull;
            uint64_t x = z;
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
            v = x ^ (x >> 31);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform integer in [0, n)
    int below(int n) { return (int)((next() >> 11) % (uint64_t)n); }
    // uniform double in (0, 1]
    double unit() { return ((next() >> 11) + 1) * (1.0 / 9007199254740992.0); }
    double gauss() {
        const double u1 = unit(), u2 = unit();
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
};

int round_half_away(double v) { return v < 0 ? -(int)floor(-v + 0.5) : (int)floor(v + 0.5); }
int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

double srgb_to_linear(double c) { return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4); }
double lab_f(double t) { return t > 216.0 / 24389.0 ? cbrt(t) : (24389.0 / 27.0 * t + 16.0) / 116.0; }

}  // namespace

extern "C" {

rts_status rts_synth_pair(uint64_t seed, int W, int H, int max_disp, int n_rects, int n_planes, float sigma,
                          int bg_disp, uint8_t *left, uint8_t *right, uint8_t *gt) {
    if (W <= 0 || H <= 0 || max_disp <= 0 || max_disp > 256 || !left || !right || n_rects < 0 || n_planes < 0)
        return RTS_ERR_INVALID_ARG;
    Rng rng(seed);
    const size_t np = (size_t)W * H;
    // texture: uniform u8, then 3x3 box (sum+4)/9 with clamp-to-edge
    std::vector<uint8_t> raw(np);
    for (auto &v : raw) v = (uint8_t)(rng.next() >> 56);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int s = 0;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++)
                    s += raw[(size_t)clampi(y + dy, 0, H - 1) * W + clampi(x + dx, 0, W - 1)];
            left[(size_t)y * W + x] = (uint8_t)((s + 4) / 9);
        }
    // disparity map on the right image's grid
    std::vector<uint8_t> d(np, (uint8_t)clampi(bg_disp, 0, max_disp - 1));
    for (int i = 0; i < n_rects; i++) {
        const int rw = 1 + rng.below(W / 3 > 1 ? W / 3 : 1), rh = 1 + rng.below(H / 3 > 1 ? H / 3 : 1);
        const int x0 = rng.below(W), y0 = rng.below(H), dv = rng.below(max_disp);
        for (int y = y0; y < y0 + rh && y < H; y++)
            for (int x = x0; x < x0 + rw && x < W; x++) d[(size_t)y * W + x] = (uint8_t)dv;
    }
    for (int i = 0; i < n_planes; i++) {
        // slanted plane d = round(a + b x + c y) over a random rectangle, clipped
        const int rw = 1 + rng.below(W / 2 > 1 ? W / 2 : 1), rh = 1 + rng.below(H / 2 > 1 ? H / 2 : 1);
        const int x0 = rng.below(W), y0 = rng.below(H);
        const double a = rng.below(max_disp);
        const double b = (rng.unit() - 0.5) * 2.0 * (double)max_disp / (double)W;
        const double c = (rng.unit() - 0.5) * 2.0 * (double)max_disp / (double)H;
        for (int y = y0; y < y0 + rh && y < H; y++)
            for (int x = x0; x < x0 + rw && x < W; x++)
                d[(size_t)y * W + x] = (uint8_t)clampi(round_half_away(a + b * (x - x0) + c * (y - y0)), 0, max_disp - 1);
    }
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const int dv = d[(size_t)y * W + x];
            const double v = left[(size_t)y * W + clampi(x + dv, 0, W - 1)] + (sigma > 0 ? sigma * rng.gauss() : 0.0);
            right[(size_t)y * W + x] = (uint8_t)clampi(round_half_away(v), 0, 255);
        }
    if (gt) memcpy(gt, d.data(), np);
    return RTS_OK;
}

void rts_gray_to_rgb(const uint8_t *gray, uint8_t *rgb, int W, int H) {
    const size_t np = (size_t)W * H;
    for (size_t i = 0; i < np; i++) rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = gray[i];
}

void rts_rgb_to_lab(const uint8_t *rgb, uint8_t *lab, int W, int H) {
    // sRGB (D65) -> XYZ -> CIE L*a*b*, 8-bit encoding L*255/100, a+128, b+128
    const size_t np = (size_t)W * H;
    for (size_t i = 0; i < np; i++) {
        const double r = srgb_to_linear(rgb[3 * i] / 255.0), g = srgb_to_linear(rgb[3 * i + 1] / 255.0),
                     b = srgb_to_linear(rgb[3 * i + 2] / 255.0);
        const double X = (0.4124564 * r + 0.3575761 * g + 0.1804375 * b) / 0.95047;
        const double Y = 0.2126729 * r + 0.7151522 * g + 0.0721750 * b;
        const double Z = (0.0193339 * r + 0.1191920 * g + 0.9503041 * b) / 1.08883;
        const double fx = lab_f(X), fy = lab_f(Y), fz = lab_f(Z);
        const double L = 116.0 * fy - 16.0, A = 500.0 * (fx - fy), B = 200.0 * (fy - fz);
        lab[3 * i] = (uint8_t)clampi(round_half_away(L * 255.0 / 100.0), 0, 255);
        lab[3 * i + 1] = (uint8_t)clampi(round_half_away(A + 128.0), 0, 255);
        lab[3 * i + 2] = (uint8_t)clampi(round_half_away(B + 128.0), 0, 255);
    }
}

}  // extern "C"
