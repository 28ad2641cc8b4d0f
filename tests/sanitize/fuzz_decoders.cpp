// Mutation driver for the library's host decoders, built by the test with
// AddressSanitizer and UndefinedBehaviorSanitizer: every mutated input must
// decode or fail with a status, with no invalid memory access.
//   fuzz_decoders <kind> <iterations> <seed file> [mode filter count stride]
// kind: png, jpeg, dds, ktx2, zstd, gltf (the seed file's extension is kept),
// meshopt (the extra arguments describe the stream).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <random>
#include <string>
#include <vector>

#include "vkgv.h"

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    const std::string kind = argv[1], path = argv[3];
    const int iterations = std::atoi(argv[2]);
    std::ifstream in(path, std::ios::binary);
    const std::vector<uint8_t> seed((std::istreambuf_iterator<char>(in)), {});
    if (seed.empty()) return 2;
    uint32_t mode = 0, filter = 0, count = 0, stride = 0;
    if (kind == "meshopt") {
        if (argc < 8) return 2;
        mode = uint32_t(std::atoi(argv[4]));
        filter = uint32_t(std::atoi(argv[5]));
        count = uint32_t(std::atoi(argv[6]));
        stride = uint32_t(std::atoi(argv[7]));
    }
    const std::string mut = path + ".mut" + path.substr(path.rfind('.'));
    std::mt19937 rng(1234);
    long ok = 0;
    for (int it = 0; it < iterations; ++it) {
        std::vector<uint8_t> m = seed;
        uint32_t n_count = count, n_stride = stride;
        if (it) {
            const int edits = 1 + int(rng() % 4);
            for (int e = 0; e < edits && !m.empty(); ++e) {
                switch (rng() % 5) {
                    case 0: m[rng() % m.size()] = uint8_t(rng()); break;
                    case 1: m[rng() % m.size()] ^= uint8_t(1u << (rng() % 8)); break;
                    case 2: m.resize(rng() % m.size()); break;
                    case 3: {  // JSON structure characters
                        static const char kChars[] = "0123456789[]{}\\\",:";
                        const size_t at = rng() % m.size();
                        for (size_t q = 0; q < 4 && at + q < m.size(); ++q) m[at + q] = uint8_t(kChars[rng() % 18]);
                        break;
                    }
                    default:
                        if (kind == "meshopt") {
                            if (rng() % 2) n_count = uint32_t(rng() % (2 * count + 8));
                            else n_stride = 1 + uint32_t(rng() % 64);
                        } else {
                            const size_t at = rng() % m.size();
                            m.insert(m.begin() + long(at), uint8_t(rng()));
                        }
                }
            }
        }
        char err[256];
        int rc = VKGV_INVALID_ARG;
        if (kind == "png") {
            vkgv_image* img = nullptr;
            rc = vkgv_image_decode_png(m.data(), m.size(), &img, err, sizeof err);
            if (rc == VKGV_OK) vkgv_image_free(img);
        } else if (kind == "jpeg") {
            vkgv_jpeg* j = nullptr;
            rc = vkgv_jpeg_decode_coefficients(m.data(), m.size(), &j, err, sizeof err);
            if (rc == VKGV_OK) vkgv_jpeg_free(j);
        } else if (kind == "dds" || kind == "ktx2") {
            vkgv_dds_info info;
            rc = kind == "dds" ? vkgv_dds_parse(m.data(), m.size(), &info) : vkgv_ktx2_parse(m.data(), m.size(), &info);
        } else if (kind == "zstd") {
            std::vector<uint8_t> out(rng() % 2 ? (1u << 20) : rng() % 4096);
            uint64_t n = 0;
            rc = vkgv_zstd_decompress(m.data(), m.size(), out.data(), out.size(), &n);
        } else if (kind == "meshopt") {
            std::vector<uint8_t> dst(size_t(n_count) * n_stride + 1);
            rc = vkgv_meshopt_decode(dst.data(), n_count, n_stride, m.data(), m.size(), int(mode), int(filter));
        } else if (kind == "gltf") {
            std::ofstream o(mut, std::ios::binary);
            o.write(reinterpret_cast<const char*>(m.data()), std::streamsize(m.size()));
            o.close();
            vkgv_gltf* g = nullptr;
            rc = vkgv_gltf_load(mut.c_str(), 0, &g, err, sizeof err);
            if (rc == VKGV_OK) vkgv_gltf_free(g);
        } else {
            return 2;
        }
        if (rc == VKGV_OK) ++ok;
        else if (rc != VKGV_INVALID_ARG && rc != VKGV_LIMIT_EXCEEDED && rc != VKGV_OUT_OF_MEMORY) {
            std::fprintf(stderr, "unexpected status %d\n", rc);
            return 3;
        }
    }
    std::printf("%d %ld\n", iterations, ok);
    return 0;
}
