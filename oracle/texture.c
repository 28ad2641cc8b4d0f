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

/* ------------------------------------------------------------------ BC7
 * BC7 (BPTC UNORM), restated from the published format: the mode from the
 * lowest set bit of the first byte; per mode the subset count, partition
 * bits, rotation and index-selection bits, colour / alpha endpoint bits,
 * p-bits (per endpoint or shared per subset) and one or two index sets;
 * endpoints expanded to 8 bits by replicating their top bits; texels
 * interpolated as ((64 - w) e0 + w e1 + 32) >> 6 with the 2-, 3- and 4-bit
 * weight tables; the anchor texel of each subset stores one index bit less.
 * A reserved mode (first byte 0) decodes to transparent black.  The
 * partition and anchor tables below are the format's own. */
static const uint16_t kBc7P2[64] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80, 0xE800,
    0xFFE8, 0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310, 0x3100, 0x8CCE,
    0x088C, 0x3110, 0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C, 0xAAAA, 0xF0F0, 0x5A5A, 0x33CC,
    0x3C3C, 0x55AA, 0x9696, 0xA55A, 0x73CE, 0x13C8, 0x324C, 0x3BDC, 0x6996, 0xC33C, 0x9966, 0x0660,
    0x0272, 0x04E4, 0x4E40, 0x2720, 0xC936, 0x936C, 0x39C6, 0x639C, 0x9336, 0x9CC6, 0x817E, 0xE718,
    0xCCF0, 0x0FCC, 0x7744, 0xEE22};
/* 3-subset partitions: two bits per texel, texel 0 in the lowest bits */
static const uint32_t kBc7P3[64] = {
    0xAA685050, 0x6A5A5040, 0x5A5A4200, 0x5450A0A8, 0xA5A50000, 0xA0A05050, 0x5555A0A0, 0x5A5A5050,
    0xAA550000, 0xAA555500, 0xAAAA5500, 0x90909090, 0x94949494, 0xA4A4A4A4, 0xA9A59450, 0x2A0A4250,
    0xA5945040, 0x0A425054, 0xA5A5A500, 0x55A0A0A0, 0xA8A85454, 0x6A6A4040, 0xA4A45000, 0x1A1A0500,
    0x0050A4A4, 0xAAA59090, 0x14696914, 0x69691400, 0xA08585A0, 0xAA821414, 0x50A4A450, 0x6A5A0200,
    0xA9A58000, 0x5090A0A8, 0xA8A09050, 0x24242424, 0x00AA5500, 0x24924924, 0x24499224, 0x50A50A50,
    0x500AA550, 0xAAAA4444, 0x66660000, 0xA5A0A5A0, 0x50A050A0, 0x69286928, 0x44AAAA44, 0x66666600,
    0xAA444444, 0x54A854A8, 0x95809580, 0x96969600, 0xA85454A8, 0x80959580, 0xAA141414, 0x96960000,
    0xAAAA1414, 0xA05050A0, 0xA0A5A5A0, 0x96000000, 0x40804080, 0xA9A8A9A8, 0xAAAAAA44, 0x2A4A5254};
static const uint8_t kBc7A2[64] = {
    15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2, 8, 2, 2, 8, 8, 15, 2, 8,
    2, 2, 8, 8, 2, 2, 15, 15, 6, 8, 2, 8, 15, 15, 2, 8, 2, 2, 2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2,
    2, 15, 15, 15, 15, 15, 2, 2, 15};
static const uint8_t kBc7A3a[64] = {
    3, 3, 15, 15, 8, 3, 15, 15, 8, 8, 6, 6, 6, 5, 3, 3, 3, 3, 8, 15, 3, 3, 6, 10, 5, 8, 8, 6, 8, 5,
    15, 15, 8, 15, 3, 5, 6, 10, 8, 15, 15, 3, 15, 5, 15, 15, 15, 15, 3, 15, 5, 5, 5, 8, 5, 10, 5,
    10, 8, 13, 15, 12, 3, 3};
static const uint8_t kBc7A3b[64] = {
    15, 8, 8, 3, 15, 15, 3, 8, 15, 15, 15, 15, 15, 15, 15, 8, 15, 8, 15, 3, 15, 8, 15, 8, 3, 15, 6,
    10, 15, 15, 10, 8, 15, 3, 15, 10, 10, 8, 9, 10, 6, 15, 8, 15, 3, 6, 6, 8, 15, 3, 15, 15, 15, 15,
    15, 15, 15, 15, 15, 15, 3, 15, 15, 8};

static const uint8_t kBc7W2[4] = {0, 21, 43, 64};
static const uint8_t kBc7W3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
static const uint8_t kBc7W4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

/* mode parameters: subsets, partition bits, rotation bits, index-selection
 * bit, colour bits, alpha bits, p-bits per endpoint, shared p-bits, index
 * bits, second index bits */
static const uint8_t kBc7Mode[8][10] = {
    {3, 4, 0, 0, 4, 0, 1, 0, 3, 0}, {2, 6, 0, 0, 6, 0, 0, 1, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 0, 2, 0},
    {2, 6, 0, 0, 7, 0, 1, 0, 2, 0}, {1, 0, 2, 1, 5, 6, 0, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 0, 2, 2},
    {1, 0, 0, 0, 7, 7, 1, 0, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 0, 2, 0}};

static uint32_t bc7_bits(const uint8_t* b, unsigned* pos, unsigned n) {
    uint32_t v = 0;
    for (unsigned i = 0; i < n; ++i, ++*pos) v |= (uint32_t)((b[*pos >> 3] >> (*pos & 7)) & 1u) << i;
    return v;
}

static unsigned bc7_expand(unsigned v, unsigned bits) {
    v <<= 8 - bits;
    return v | (v >> bits);
}

static unsigned bc7_interp(unsigned e0, unsigned e1, unsigned w) { return ((64 - w) * e0 + w * e1 + 32) >> 6; }

static void bc7_block(const uint8_t* b, uint32_t out[16]) {
    unsigned mode = 0;
    while (mode < 8 && !((b[0] >> mode) & 1u)) ++mode;
    if (mode == 8) {
        for (int i = 0; i < 16; ++i) out[i] = 0;
        return;
    }
    const uint8_t* m = kBc7Mode[mode];
    const unsigned ns = m[0], cb = m[4], ab = m[5], ib = m[8], ib2 = m[9];
    unsigned pos = mode + 1;
    const unsigned part = bc7_bits(b, &pos, m[1]);
    const unsigned rot = bc7_bits(b, &pos, m[2]);
    const unsigned isel = bc7_bits(b, &pos, m[3]);
    unsigned ep[3][2][4]; /* subset, endpoint, channel */
    for (unsigned c = 0; c < 3; ++c)
        for (unsigned s = 0; s < ns; ++s)
            for (unsigned e = 0; e < 2; ++e) ep[s][e][c] = bc7_bits(b, &pos, cb);
    for (unsigned s = 0; s < ns; ++s)
        for (unsigned e = 0; e < 2; ++e) ep[s][e][3] = ab ? bc7_bits(b, &pos, ab) : 255u;
    unsigned cbits = cb, abits = ab;
    if (m[6]) { /* a p-bit per endpoint */
        for (unsigned s = 0; s < ns; ++s)
            for (unsigned e = 0; e < 2; ++e) {
                const unsigned p = bc7_bits(b, &pos, 1);
                for (unsigned c = 0; c < 4; ++c)
                    if (c < 3 || ab) ep[s][e][c] = (ep[s][e][c] << 1) | p;
            }
        cbits = cb + 1;
        abits = ab ? ab + 1 : 0;
    } else if (m[7]) { /* a p-bit per subset */
        for (unsigned s = 0; s < ns; ++s) {
            const unsigned p = bc7_bits(b, &pos, 1);
            for (unsigned e = 0; e < 2; ++e)
                for (unsigned c = 0; c < 3; ++c) ep[s][e][c] = (ep[s][e][c] << 1) | p;
        }
        cbits = cb + 1;
    }
    for (unsigned s = 0; s < ns; ++s)
        for (unsigned e = 0; e < 2; ++e) {
            for (unsigned c = 0; c < 3; ++c) ep[s][e][c] = bc7_expand(ep[s][e][c], cbits);
            if (ab) ep[s][e][3] = bc7_expand(ep[s][e][3], abits);
        }
    /* subset of each texel and the anchors (texel 0 for subset 0) */
    unsigned sub[16], anchor[3] = {0, 16, 16};
    for (unsigned i = 0; i < 16; ++i)
        sub[i] = ns == 1 ? 0u : (ns == 2 ? ((kBc7P2[part] >> i) & 1u) : ((kBc7P3[part] >> (2 * i)) & 3u));
    if (ns == 2) anchor[1] = kBc7A2[part];
    if (ns == 3) {
        anchor[1] = kBc7A3a[part];
        anchor[2] = kBc7A3b[part];
    }
    unsigned idx[16], idx2[16];
    for (unsigned i = 0; i < 16; ++i) {
        const int is_anchor = i == anchor[0] || i == anchor[1] || i == anchor[2];
        idx[i] = bc7_bits(b, &pos, ib - (is_anchor ? 1u : 0u));
    }
    for (unsigned i = 0; ib2 && i < 16; ++i) idx2[i] = bc7_bits(b, &pos, ib2 - (i == 0 ? 1u : 0u));
    for (unsigned i = 0; i < 16; ++i) {
        const unsigned s = sub[i];
        unsigned ci = idx[i], ai = idx[i], cw_bits = ib, aw_bits = ib;
        if (ib2) {
            if (isel) {
                ci = idx2[i], cw_bits = ib2;
            } else {
                ai = idx2[i], aw_bits = ib2;
            }
        }
        const uint8_t* cw = cw_bits == 2 ? kBc7W2 : (cw_bits == 3 ? kBc7W3 : kBc7W4);
        const uint8_t* aw = aw_bits == 2 ? kBc7W2 : (aw_bits == 3 ? kBc7W3 : kBc7W4);
        unsigned px[4];
        for (unsigned c = 0; c < 3; ++c) px[c] = bc7_interp(ep[s][0][c], ep[s][1][c], cw[ci]);
        px[3] = ab ? bc7_interp(ep[s][0][3], ep[s][1][3], aw[ai]) : 255u;
        if (rot) { /* swap alpha with R (1), G (2) or B (3) */
            const unsigned t = px[3];
            px[3] = px[rot - 1];
            px[rot - 1] = t;
        }
        out[i] = px[0] | (px[1] << 8) | (px[2] << 16) | (px[3] << 24);
    }
}

void orc_decode_bc(uint32_t format, const uint8_t* blocks, uint32_t w, uint32_t h, uint32_t* rgba) {
    uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    size_t bsize = (format == 1 || format == 4 || format == 6) ? 8 : 16; /* 8: BC7 */
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
                case 8:
                    bc7_block(p, tex);
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

/* ------------------------------------------------------------------ BC6H
 * BC6H (BPTC float; UF16 unsigned, SF16 signed), restated from the published
 * format: a 2-bit mode (values 0, 1) or a 5-bit one; fourteen modes of one or
 * two regions whose 77-80 header bits hold the endpoint channels in a
 * mode-specific order (the token tables below; three modes store the top
 * bits of their base endpoint reversed) and, for two regions, a 5-bit
 * partition (the first 32 two-subset partitions of BC7, with their
 * anchors).  Transformed modes store the other endpoints as signed deltas
 * from the base, added and wrapped to the endpoint precision (then sign-
 * extended for SF16); untransformed SF16 endpoints are sign-extended.
 * Endpoints are unquantised to 16 bits (unsigned: 0 and the top code map to
 * 0 and 0xFFFF, others to ((c << 16) + 0x8000) >> bits; signed: on the
 * magnitude, 0x7FFF from 2^(bits-1) - 1 up, ((c << 15) + 0x4000) >> (bits-1)
 * otherwise), texels interpolated as ((64 - w) e0 + w e1 + 32) >> 6 with the
 * 3-bit (two regions) or 4-bit weights (the anchors store one index bit
 * less), and scaled into binary16 bits: unsigned v * 31 >> 6; signed the
 * magnitude * 31 >> 5, the sign bit set only on a non-zero result.
 * Reserved modes decode to 0.  Matches the GPU texture unit's BC6H decode bit
 * for bit on every mode (tests/golden/bc6h_texture_unit.json). */

/* header tokens: field (bits 0-3: endpoint w, x, y, z x channel R, G, B, or
 * 12 = partition), lowest field bit (4-7), bit count - 1 (8-11), reversed
 * (12: the first stream bit is the highest field bit) */
static const uint16_t kBc6Tok[14][23] = {
    {0x0047, 0x0048, 0x004B, 0x0900, 0x0901, 0x0902, 0x0403, 0x004A, 0x0307, 0x0404, 0x000B, 0x030A, 0x0405, 0x001B, 0x0308, 0x0406, 0x002B, 0x0409, 0x003B, 0x040C},  /* mode 0x00 */
    {0x0057, 0x014A, 0x0600, 0x010B, 0x0048, 0x0601, 0x0058, 0x002B, 0x0047, 0x0602, 0x003B, 0x005B, 0x004B, 0x0503, 0x0307, 0x0504, 0x030A, 0x0505, 0x0308, 0x0506, 0x0509, 0x040C},  /* mode 0x01 */
    {0x0900, 0x0901, 0x0902, 0x0403, 0x00A0, 0x0307, 0x0304, 0x00A1, 0x000B, 0x030A, 0x0305, 0x00A2, 0x001B, 0x0308, 0x0406, 0x002B, 0x0409, 0x003B, 0x040C},  /* mode 0x02 */
    {0x0900, 0x0901, 0x0902, 0x0303, 0x00A0, 0x004A, 0x0307, 0x0404, 0x00A1, 0x030A, 0x0305, 0x00A2, 0x001B, 0x0308, 0x0306, 0x000B, 0x002B, 0x0309, 0x0047, 0x003B, 0x040C},  /* mode 0x06 */
    {0x0900, 0x0901, 0x0902, 0x0303, 0x00A0, 0x0048, 0x0307, 0x0304, 0x00A1, 0x000B, 0x030A, 0x0405, 0x00A2, 0x0308, 0x0306, 0x011B, 0x0309, 0x004B, 0x003B, 0x040C},  /* mode 0x0A */
    {0x0800, 0x0048, 0x0801, 0x0047, 0x0802, 0x004B, 0x0403, 0x004A, 0x0307, 0x0404, 0x000B, 0x030A, 0x0405, 0x001B, 0x0308, 0x0406, 0x002B, 0x0409, 0x003B, 0x040C},  /* mode 0x0E */
    {0x0700, 0x004A, 0x0048, 0x0701, 0x002B, 0x0047, 0x0702, 0x013B, 0x0503, 0x0307, 0x0404, 0x000B, 0x030A, 0x0405, 0x001B, 0x0308, 0x0506, 0x0509, 0x040C},  /* mode 0x12 */
    {0x0700, 0x000B, 0x0048, 0x0701, 0x0057, 0x0047, 0x0702, 0x005A, 0x004B, 0x0403, 0x004A, 0x0307, 0x0504, 0x030A, 0x0405, 0x001B, 0x0308, 0x0406, 0x002B, 0x0409, 0x003B, 0x040C},  /* mode 0x16 */
    {0x0700, 0x001B, 0x0048, 0x0701, 0x0058, 0x0047, 0x0702, 0x005B, 0x004B, 0x0403, 0x004A, 0x0307, 0x0404, 0x000B, 0x030A, 0x0505, 0x0308, 0x0406, 0x002B, 0x0409, 0x003B, 0x040C},  /* mode 0x1A */
    {0x0500, 0x004A, 0x010B, 0x0048, 0x0501, 0x0057, 0x0058, 0x002B, 0x0047, 0x0502, 0x005A, 0x003B, 0x005B, 0x004B, 0x0503, 0x0307, 0x0504, 0x030A, 0x0505, 0x0308, 0x0506, 0x0509, 0x040C},  /* mode 0x1E */
    {0x0900, 0x0901, 0x0902, 0x0903, 0x0904, 0x0905},  /* mode 0x03 */
    {0x0900, 0x0901, 0x0902, 0x0803, 0x00A0, 0x0804, 0x00A1, 0x0805, 0x00A2},  /* mode 0x07 */
    {0x0900, 0x0901, 0x0902, 0x0703, 0x11A0, 0x0704, 0x11A1, 0x0705, 0x11A2},  /* mode 0x0B */
    {0x0900, 0x0901, 0x0902, 0x0303, 0x15A0, 0x0304, 0x15A1, 0x0305, 0x15A2},  /* mode 0x0F */
};
/* mode value, transformed, endpoint bits, delta bits R, G, B, regions, tokens */
static const uint8_t kBc6Mode[14][8] = {
    {0x00, 1, 10, 5, 5, 5, 2, 20},
    {0x01, 1, 7, 6, 6, 6, 2, 22},
    {0x02, 1, 11, 5, 4, 4, 2, 19},
    {0x06, 1, 11, 4, 5, 4, 2, 21},
    {0x0A, 1, 11, 4, 4, 5, 2, 20},
    {0x0E, 1, 9, 5, 5, 5, 2, 20},
    {0x12, 1, 8, 6, 5, 5, 2, 19},
    {0x16, 1, 8, 5, 6, 5, 2, 22},
    {0x1A, 1, 8, 5, 5, 6, 2, 22},
    {0x1E, 0, 6, 6, 6, 6, 2, 23},
    {0x03, 0, 10, 10, 10, 10, 1, 6},
    {0x07, 1, 11, 9, 9, 9, 1, 9},
    {0x0B, 1, 12, 8, 8, 8, 1, 9},
    {0x0F, 1, 16, 4, 4, 4, 1, 9}};

static int32_t bc6_sext(uint32_t v, unsigned n) {
    v &= (n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u));
    return (v >> (n - 1)) & 1u ? (int32_t)v - (int32_t)(1u << n) : (int32_t)v;
}

static int32_t bc6_unquantize(int32_t c, unsigned bits, int sgn) {
    if (!sgn) {
        if (bits >= 15) return c;
        if (c == 0) return 0;
        if (c == (int32_t)((1u << bits) - 1u)) return 0xFFFF;
        return (int32_t)((((uint32_t)c << 16) + 0x8000u) >> bits);
    }
    if (bits >= 16) return c;
    const int neg = c < 0;
    int32_t m = neg ? -c : c, u;
    if (m == 0)
        u = 0;
    else if (m >= (int32_t)((1u << (bits - 1)) - 1u))
        u = 0x7FFF;
    else
        u = (int32_t)((((uint32_t)m << 15) + 0x4000u) >> (bits - 1));
    return neg ? -u : u;
}

/* floor(v / 64) */
static int32_t bc6_asr6(int32_t v) { return v >= 0 ? v >> 6 : -((-v - 1) >> 6) - 1; }

static uint16_t bc6_finish(int32_t v, int sgn) {
    if (!sgn) return (uint16_t)((v * 31) >> 6);
    if (v < 0) {
        const int32_t m = ((-v) * 31) >> 5;
        return (uint16_t)(m ? (m | 0x8000) : 0);
    }
    return (uint16_t)((v * 31) >> 5);
}

static void bc6_block(const uint8_t* b, int sgn, uint16_t out[16][3]) {
    unsigned pos = 0;
    unsigned m = bc7_bits(b, &pos, 2);
    if (m >= 2) m |= bc7_bits(b, &pos, 3) << 2;
    int mi = -1;
    for (int i = 0; i < 14; ++i)
        if (kBc6Mode[i][0] == m) mi = i;
    if (mi < 0) {
        for (int i = 0; i < 16; ++i) out[i][0] = out[i][1] = out[i][2] = 0;
        return;
    }
    const uint8_t* M = kBc6Mode[mi];
    uint32_t f[13] = {0};
    for (unsigned t = 0; t < M[7]; ++t) {
        const unsigned tok = kBc6Tok[mi][t], fid = tok & 15u, lo = (tok >> 4) & 15u, n = ((tok >> 8) & 15u) + 1u;
        uint32_t v = bc7_bits(b, &pos, n);
        if (tok >> 12) {
            uint32_t r = 0;
            for (unsigned k = 0; k < n; ++k) r |= ((v >> k) & 1u) << (n - 1u - k);
            v = r;
        }
        f[fid] |= v << lo;
    }
    const unsigned tr = M[1], bits = M[2], ns = M[6];
    int32_t ep[4][3];
    for (unsigned e = 0; e < 2 * ns; ++e)
        for (unsigned c = 0; c < 3; ++c) {
            const uint32_t raw = f[e * 3 + c];
            int32_t v;
            if (e == 0 || !tr) {
                v = sgn ? bc6_sext(raw, bits) : (int32_t)raw;
            } else {
                const int32_t d = bc6_sext(raw, M[3 + c]);
                const uint32_t sum = (uint32_t)((int32_t)f[c] + d) & ((1u << bits) - 1u);
                v = sgn ? bc6_sext(sum, bits) : (int32_t)sum;
            }
            ep[e][c] = bc6_unquantize(v, bits, sgn);
        }
    const unsigned part = f[12] & 31u, anchor = ns == 2 ? kBc7A2[part] : 16u, ib = ns == 2 ? 3u : 4u;
    for (unsigned i = 0; i < 16; ++i) {
        const unsigned idx = bc7_bits(b, &pos, ib - ((i == 0 || i == anchor) ? 1u : 0u));
        const unsigned s = ns == 2 ? ((kBc7P2[part] >> i) & 1u) : 0u;
        const int32_t w = ns == 2 ? kBc7W3[idx] : kBc7W4[idx];
        for (unsigned c = 0; c < 3; ++c)
            out[i][c] = bc6_finish(bc6_asr6((64 - w) * ep[2 * s][c] + w * ep[2 * s + 1][c] + 32), sgn);
    }
}

void orc_decode_bc6h(const uint8_t* blocks, uint32_t w, uint32_t h, int is_signed, uint16_t* rgb) {
    const uint32_t bw = (w + 3) / 4, bh = (h + 3) / 4;
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            uint16_t tex[16][3];
            bc6_block(blocks + ((size_t)by * bw + bx) * 16, is_signed, tex);
            for (int i = 0; i < 16; ++i) {
                const uint32_t x = bx * 4 + (uint32_t)(i % 4), y = by * 4 + (uint32_t)(i / 4);
                if (x < w && y < h)
                    for (int c = 0; c < 3; ++c) rgb[((size_t)y * w + x) * 3 + c] = tex[i][c];
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
