/*
 * texture.c: CPU restatement of the block-compressed texture formats
 * (BC1-BC5, the DXT1-5 / RGTC layouts of DDS files) decoded into RGBA8.
 * TEST INFRASTRUCTURE ONLY: the parity tests call it as the checker.
 *
 * The reference decodes no images (src/vk_gltf_viewer/assets.cpp:467-471),
 * so parity is with the published formats.  Their interpolation rounding is
 * implementation-defined and pinned as (integer arithmetic):
 *   565 -> 888 by bit replication;
 *   four-colour blocks: (2 c0 + c1 + 1) / 3 and (c0 + 2 c1 + 1) / 3;
 *   BC1 three-colour blocks (c0 <= c1): (c0 + c1 + 1) / 2, then transparent black;
 *   BC2 alpha: 4-bit value * 17;
 *   8-value channel blocks (a0 > a1): ((7 - j) a0 + j a1 + 3) / 7, j = 1..6;
 *   6-value channel blocks: ((5 - j) a0 + j a1 + 2) / 5, j = 1..4, then 0 and 255.
 * BC4 gives (r, 0, 0, 255), BC5 (r, g, 0, 255).  Format 6 is BC1 read as
 * Vulkan's BC1_RGB formats: the three-colour mode's fourth entry is opaque
 * black.
 */
#include "oracle.h"

#include <string.h>

static void expand565(unsigned c, unsigned out[3]) {
    unsigned r = (c >> 11) & 31u, g = (c >> 5) & 63u, b = c & 31u;
    out[0] = (r << 3) | (r >> 2);
    out[1] = (g << 2) | (g >> 4);
    out[2] = (b << 3) | (b >> 2);
}

/* The 16 RGBA texels of a BC1-layout colour block; three_allowed = 2 is
 * BC1 read as Vulkan's BC1_RGB formats (the fourth three-mode entry is
 * opaque black). */
static void colour_block(const uint8_t* p, int three_allowed, uint32_t out[16]) {
    unsigned c0 = p[0] | (p[1] << 8), c1 = p[2] | (p[3] << 8);
    unsigned pal[4][4];
    unsigned a[3], b[3];
    expand565(c0, a);
    expand565(c1, b);
    int four = !three_allowed || c0 > c1;
    for (int k = 0; k < 3; ++k) {
        pal[0][k] = a[k];
        pal[1][k] = b[k];
        if (four) {
            pal[2][k] = (2 * a[k] + b[k] + 1) / 3;
            pal[3][k] = (a[k] + 2 * b[k] + 1) / 3;
        } else {
            pal[2][k] = (a[k] + b[k] + 1) / 2;
            pal[3][k] = 0;
        }
    }
    pal[0][3] = pal[1][3] = pal[2][3] = 255;
    pal[3][3] = (four || three_allowed == 2) ? 255 : 0;
    uint32_t bits = (uint32_t)p[4] | ((uint32_t)p[5] << 8) | ((uint32_t)p[6] << 16) | ((uint32_t)p[7] << 24);
    for (int i = 0; i < 16; ++i) {
        unsigned c = (bits >> (2 * i)) & 3u;
        out[i] = pal[c][0] | (pal[c][1] << 8) | (pal[c][2] << 16) | ((uint32_t)pal[c][3] << 24);
    }
}

/* The 16 values of an 8-byte interpolated channel block (BC3 alpha, BC4). */
static void channel_block(const uint8_t* p, unsigned out[16]) {
    unsigned a0 = p[0], a1 = p[1], pal[8];
    pal[0] = a0;
    pal[1] = a1;
    if (a0 > a1) {
        for (unsigned j = 1; j <= 6; ++j) pal[j + 1] = ((7 - j) * a0 + j * a1 + 3) / 7;
    } else {
        for (unsigned j = 1; j <= 4; ++j) pal[j + 1] = ((5 - j) * a0 + j * a1 + 2) / 5;
        pal[6] = 0;
        pal[7] = 255;
    }
    uint64_t bits = 0;
    for (int k = 0; k < 6; ++k) bits |= (uint64_t)p[2 + k] << (8 * k);
    for (int i = 0; i < 16; ++i) out[i] = pal[(bits >> (3 * i)) & 7u];
}

void orc_decode_bc(uint32_t format, const uint8_t* blocks, uint32_t w, uint32_t h, uint32_t* rgba) {
    uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    size_t bsize = (format == 1 || format == 4 || format == 6) ? 8 : 16;
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            const uint8_t* p = blocks + ((size_t)by * bw + bx) * bsize;
            uint32_t tex[16];
            uint32_t col[16];
            unsigned ch0[16], ch1[16];
            switch (format) {
                case 1:
                    colour_block(p, 1, tex);
                    break;
                case 6:
                    colour_block(p, 2, tex);
                    break;
                case 2:
                    colour_block(p + 8, 0, col);
                    for (int i = 0; i < 16; ++i) {
                        unsigned a4 = (p[i / 2] >> ((i % 2) * 4)) & 15u;
                        tex[i] = (col[i] & 0x00FFFFFFu) | ((uint32_t)(a4 * 17) << 24);
                    }
                    break;
                case 3:
                    colour_block(p + 8, 0, col);
                    channel_block(p, ch0);
                    for (int i = 0; i < 16; ++i) tex[i] = (col[i] & 0x00FFFFFFu) | ((uint32_t)ch0[i] << 24);
                    break;
                case 4:
                    channel_block(p, ch0);
                    for (int i = 0; i < 16; ++i) tex[i] = ch0[i] | 0xFF000000u;
                    break;
                default:
                    channel_block(p, ch0);
                    channel_block(p + 8, ch1);
                    for (int i = 0; i < 16; ++i) tex[i] = ch0[i] | (ch1[i] << 8) | 0xFF000000u;
            }
            for (int i = 0; i < 16; ++i) {
                uint32_t x = bx * 4 + (uint32_t)(i % 4), y = by * 4 + (uint32_t)(i / 4);
                if (x < w && y < h) rgba[(size_t)y * w + x] = tex[i];
            }
        }
}

/*
 * JPEG, the pixel half (the reference links wuffs for JPEG,
 * src/vk_gltf_viewer/wuffs_implementation.cpp:1-5; it is absent, so parity
 * with it is unpinned).  From dequantized natural-order coefficient blocks:
 *   the 8x8 inverse DCT, f(x, y) = sum_u sum_v c(u)/2 c(v)/2 F(v, u)
 *   cos((2x+1) u pi/16) cos((2y+1) v pi/16), c(0) = 1/sqrt(2), evaluated in
 *   the pinned fixed point: constants K[x][u] = round(8192 c(u)/2 cos(..))
 *   (derived here from the formula), the row pass rounded to 3 fractional
 *   bits ((sum + 512) >> 10), the column pass (sum + 2^15) >> 16, + 128,
 *   clamped to 0..255;
 *   chroma upsampling by replication, and the JFIF YCbCr -> RGB conversion
 *   with 16-bit fixed-point constants 1.402, 0.344136, 0.714136, 1.772
 *   (91881, 22554, 46802, 116130), rounded by + 2^15 before >> 16.
 */
#include <math.h>

static int32_t jpeg_k[8][8];
static int jpeg_k_ready;

static void jpeg_constants(void) {
    if (jpeg_k_ready) return;
    for (int x = 0; x < 8; ++x)
        for (int u = 0; u < 8; ++u) {
            const double cu = u == 0 ? 1.0 / sqrt(2.0) : 1.0;
            jpeg_k[x][u] = (int32_t)lround(8192.0 * cu / 2.0 * cos((2 * x + 1) * u * acos(-1.0) / 16.0));
        }
    jpeg_k_ready = 1;
}

static int32_t asr(int64_t v, int s) { return (int32_t)(v >= 0 ? v >> s : -((-v - 1) >> s) - 1); }

void orc_jpeg_idct(const int16_t* coef, uint32_t blocks_w, uint32_t blocks_h, uint8_t* plane) {
    jpeg_constants();
    const size_t pitch = (size_t)blocks_w * 8;
    for (uint32_t by = 0; by < blocks_h; ++by)
        for (uint32_t bx = 0; bx < blocks_w; ++bx) {
            const int16_t* F = coef + ((size_t)by * blocks_w + bx) * 64;
            int32_t t[8][8];
            for (int v = 0; v < 8; ++v)
                for (int x = 0; x < 8; ++x) {
                    int64_t sum = 0;
                    for (int u = 0; u < 8; ++u) sum += (int64_t)jpeg_k[x][u] * F[v * 8 + u];
                    t[v][x] = asr(sum + 512, 10);
                }
            for (int y = 0; y < 8; ++y)
                for (int x = 0; x < 8; ++x) {
                    int64_t sum = 0;
                    for (int v = 0; v < 8; ++v) sum += (int64_t)jpeg_k[y][v] * t[v][x];
                    int32_t s = asr(sum + 32768, 16) + 128;
                    s = s < 0 ? 0 : (s > 255 ? 255 : s);
                    plane[((size_t)by * 8 + y) * pitch + (size_t)bx * 8 + x] = (uint8_t)s;
                }
        }
}

static int32_t clamp255(int32_t v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }

void orc_jpeg_color(const uint8_t* p0, const uint8_t* p1, const uint8_t* p2, const uint32_t pitch[3],
                    const uint32_t rx[3], const uint32_t ry[3], uint32_t w, uint32_t h, uint32_t components,
                    uint32_t rgb, uint32_t* out) {
    const uint8_t* planes[3] = {p0, p1, p2};
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            int32_t c[3] = {0, 0, 0};
            for (uint32_t k = 0; k < components; ++k)
                c[k] = planes[k][(size_t)(y / ry[k]) * pitch[k] + x / rx[k]];
            int32_t r, g, b;
            if (components == 1) {
                r = g = b = c[0];
            } else if (rgb) {
                r = c[0];
                g = c[1];
                b = c[2];
            } else {
                const int32_t cb = c[1] - 128, cr = c[2] - 128;
                r = clamp255(c[0] + asr((int64_t)91881 * cr + 32768, 16));
                g = clamp255(c[0] + asr((int64_t)-22554 * cb - (int64_t)46802 * cr + 32768, 16));
                b = clamp255(c[0] + asr((int64_t)116130 * cb + 32768, 16));
            }
            out[(size_t)y * w + x] = (uint32_t)r | ((uint32_t)g << 8) | ((uint32_t)b << 16) | 0xFF000000u;
        }
}
