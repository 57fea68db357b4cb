// rts_stereo -- headless equivalent of the reference driver seq/Main.cpp.
//
// The same ten positional arguments (seq/Main.cpp:50-61):
//   1 reference image   2 target image   3 disparity range
//   4 first cost  (1 AD, 2 rank, 3 census, 4 LoG)
//   5 second cost (0 none, 1 AD, 2 rank, 3 census, 4 LoG)
//   6 aggregation (1 block, 2 adaptive weight, 3 cross-based)
//   7 scaling (0 coefficient chosen by the disparity range, 1 stretch to 255)
//   8 first lambda   9 second lambda (integers, seq/Main.cpp:85-86)
//   10 dataset name (the output is <name>_<4>_<5>_<6>_<7>_<8>_<9>.png)
// It runs the reference driver's left-view pipeline (seq/Main.cpp:180-257: the
// right view and the cross check are commented out there) with the driver's
// constants on the GPU, scales the disparity map as seq/Main.cpp:258-274 does
// and writes it.  Images are binary PGM (P5, gray: the colour image is the gray
// one in three channels, as imread(..., 1) gives for a gray file) or PPM (P6,
// RGB; its gray image is the BT.601 luma in 14-bit fixed point, the conversion
// OpenCV's imread(..., 0) applies -- OpenCV itself is not used, so this one step
// is not pinned to it).  The HighGUI preview window (seq/Main.cpp:280-282) is
// dropped.  Exit codes follow the reference: -1 for bad arguments or images, 0
// for a disparity range without a scaling coefficient, 1 after writing.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rtstereo.h"

namespace {

// ---- PGM / PPM input --------------------------------------------------------
int next_int(FILE *f) {
    int c = fgetc(f);
    for (;;) {
        while (c == ' ' || c == '\t' || c == '\n' || c == '\r') c = fgetc(f);
        if (c != '#') break;
        while (c != '\n' && c != EOF) c = fgetc(f);  // comment line
    }
    int v = 0, digits = 0;
    while (c >= '0' && c <= '9') {
        v = v * 10 + (c - '0');
        digits++;
        c = fgetc(f);
    }
    return digits ? v : -1;  // the single whitespace after the value is consumed
}

bool read_pnm(const char *path, int &W, int &H, std::vector<uint8_t> &gray, std::vector<uint8_t> &rgb) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    char magic[2] = {0, 0};
    bool ok = fread(magic, 1, 2, f) == 2 && magic[0] == 'P' && (magic[1] == '5' || magic[1] == '6');
    if (ok) {
        W = next_int(f);
        H = next_int(f);
        const int maxv = next_int(f);
        ok = W > 0 && H > 0 && maxv == 255;
    }
    if (ok) {
        const size_t np = (size_t)W * H;
        gray.resize(np);
        rgb.resize(np * 3);
        if (magic[1] == '5') {
            ok = fread(gray.data(), 1, np, f) == np;
            for (size_t i = 0; i < np; i++) rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = gray[i];
        } else {
            ok = fread(rgb.data(), 1, np * 3, f) == np * 3;
            for (size_t i = 0; i < np; i++)
                gray[i] = (uint8_t)((4899u * rgb[3 * i] + 9617u * rgb[3 * i + 1] + 1868u * rgb[3 * i + 2] + 8192u) >> 14);
        }
    }
    fclose(f);
    return ok;
}

// ---- PNG output (8-bit gray, deflate "stored" blocks: no compression library) --
uint32_t crc32_of(const uint8_t *p, size_t n, uint32_t c = 0xffffffffu) {
    static uint32_t table[256];
    static bool made = false;
    if (!made) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t v = i;
            for (int k = 0; k < 8; k++) v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            table[i] = v;
        }
        made = true;
    }
    for (size_t i = 0; i < n; i++) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c;
}

void put32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t> &out, const char *type, const std::vector<uint8_t> &data) {
    put32(out, (uint32_t)data.size());
    std::vector<uint8_t> td(type, type + 4);
    td.insert(td.end(), data.begin(), data.end());
    out.insert(out.end(), td.begin(), td.end());
    put32(out, crc32_of(td.data(), td.size()) ^ 0xffffffffu);
}

bool write_png_gray(const std::string &path, int W, int H, const uint8_t *img) {
    // scanlines with filter byte 0, wrapped in a zlib stream of stored blocks
    std::vector<uint8_t> raw;
    raw.reserve((size_t)(W + 1) * H);
    for (int y = 0; y < H; y++) {
        raw.push_back(0);
        raw.insert(raw.end(), img + (size_t)y * W, img + (size_t)(y + 1) * W);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t v : raw) {
        a = (a + v) % 65521u;
        b = (b + a) % 65521u;
    }
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t n = std::min<size_t>(65535, raw.size() - off);
        const bool last = off + n >= raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)n);
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)~n);
        z.push_back((uint8_t)(~n >> 8));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
        if (last) break;
    }
    put32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)W);
    put32(ihdr, (uint32_t)H);
    ihdr.insert(ihdr.end(), {8, 0, 0, 0, 0});  // 8-bit gray, deflate, no filter / interlace
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(png.data(), 1, png.size(), f) == png.size();
    return fclose(f) == 0 && ok;
}

// ---- seq/Main.cpp:33 round() and the scalings of :258-274 --------------------
float round_ref(float x) { return (float)(x < 0 ? std::ceil(x - 0.5) : std::floor(x + 0.5)); }

void scale_by(uint8_t *img, size_t n, float coeff) {
    for (size_t i = 0; i < n; i++) {
        float res = round_ref((float)img[i] * coeff);
        res = res > 255 ? 255 : res;
        img[i] = (uint8_t)res;
    }
}

void scale_auto(uint8_t *img, size_t n) {
    uint8_t upper = 0;
    for (size_t i = 0; i < n; i++)
        if (img[i] > upper) upper = img[i];
    scale_by(img, n, (float)255 / (float)upper);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 11) {
        printf("Need two image data and disparity range\n");
        printf("Argument 1 : Reference Image Name\n");
        printf("Argument 2 : Target Image Name\n");
        printf("Argument 3 : Disparity Range\n");
        printf("Argument 4 : First Cost Evaluation Type: (1) AD, (2) Rank, (3) Census, (4) LoG \n");
        printf("Argument 5 : Second Cost Evaluation Type: (0) Single Cost (1) AD, (2) Rank, (3) Census, (4) LoG \n");
        printf("Argument 6 : Cost Aggregation Type: (1) Block, (2) Adaptive Weight, (3) Cross-Based \n");
        printf("Argument 7 : Auto Scale or Not: (0)Scale with Pre-determined Coefficient, (1) Auto Scale \n");
        printf("Argument 8 : Coefficient of First Cost (First Lambda) \n");
        printf("Argument 9 : Coefficient of Second Cost (Second Lambda) \n");
        printf("Argument 10: Name of Dataset(Image) \n");
        return -1;
    }
    int W = 0, H = 0, W2 = 0, H2 = 0;
    std::vector<uint8_t> lg, lc, rg, rc;
    if (!read_pnm(argv[1], W, H, lg, lc) || !read_pnm(argv[2], W2, H2, rg, rc) || W != W2 || H != H2) {
        printf("incorrect image data \n");
        return -1;
    }
    rts_params p;
    rts_params_default(&p);  // the driver's constants (seq/Main.cpp:102-131)
    p.disp_range = atoi(argv[3]);
    p.cost1 = atoi(argv[4]);
    p.cost2 = atoi(argv[5]);
    p.aggr = atoi(argv[6]);
    const int auto_scale = atoi(argv[7]);
    p.lambda1 = (float)atoi(argv[8]);
    p.lambda2 = (float)atoi(argv[9]);
    p.right_view = 0;
    std::vector<uint8_t> ll, rl;
    if (p.aggr == RTS_AGGR_AW) {
        ll.resize(lc.size());
        rl.resize(rc.size());
        rts_rgb_to_lab(lc.data(), ll.data(), W, H);
        rts_rgb_to_lab(rc.data(), rl.data(), W, H);
    }
    rts_ctx *ctx = nullptr;
    if (rts_ctx_create(&ctx, 0, 0) != RTS_OK) {
        printf("ERR:no GPU context\n");
        return -1;
    }
    std::vector<uint8_t> disp((size_t)W * H);
    rts_pair pair{W, H, lg.data(), rg.data(), lc.data(), rc.data(), ll.empty() ? nullptr : ll.data(),
                  rl.empty() ? nullptr : rl.data()};
    rts_out out{disp.data(), nullptr, nullptr, nullptr};
    const rts_status st = rts_pipeline_run(ctx, RTS_HOST, &pair, &p, &out);
    if (st != RTS_OK) {
        printf("ERR:%s\n", rts_ctx_last_error(ctx));
        rts_ctx_destroy(ctx);
        return -1;
    }
    rts_ctx_destroy(ctx);
    const size_t np = disp.size();
    if (auto_scale == 1) {
        scale_auto(disp.data(), np);
    } else if (p.disp_range == 16) {
        scale_by(disp.data(), np, 16);
    } else if (p.disp_range == 20) {
        scale_by(disp.data(), np, 8);
    } else if (p.disp_range == 60) {
        scale_by(disp.data(), np, 4);
    } else {
        printf("Invalid disparity range! \n");
        return 0;
    }
    const std::string dash = "_";
    const std::string name = std::string(argv[10]) + dash + argv[4] + dash + argv[5] + dash + argv[6] + dash +
                             argv[7] + dash + argv[8] + dash + argv[9] + ".png";
    if (!write_png_gray(name, W, H, disp.data())) {
        printf("ERR:cannot write %s\n", name.c_str());
        return -1;
    }
    return 1;
}
