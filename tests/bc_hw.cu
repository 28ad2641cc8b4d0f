// A second, independent BC decoder for the block-compression parity tests:
// the GPU's own texture unit.  The blocks go into a block-compressed CUDA
// array, one thread per texel reads it through a point-sampled texture
// object, and the normalised texels come back as RGBA8 (channels a format
// lacks read as the texture unit returns them); BC6H texels come back as
// four float32 values (R, G, B, A) each.
//   bc_hw <format> <blocks.bin> <out.bin> <width> <height>
// format: the library's numbering (VKGV_BC1-VKGV_BC5 = 1-5, VKGV_BC7 = 8,
// VKGV_BC6H_UF16 = 9, VKGV_BC6H_SF16 = 10); width, height: multiples of 4.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

__global__ void k_fetch_float(cudaTextureObject_t tex, unsigned w, unsigned h, float4* out) {
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    out[(size_t)y * w + x] = tex2D<float4>(tex, x + 0.5f, y + 0.5f);
}

__global__ void k_fetch(cudaTextureObject_t tex, unsigned w, unsigned h, unsigned* out) {
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    const float4 v = tex2D<float4>(tex, x + 0.5f, y + 0.5f);
    const unsigned r = __float2uint_rn(__saturatef(v.x) * 255.0f), g = __float2uint_rn(__saturatef(v.y) * 255.0f);
    const unsigned b = __float2uint_rn(__saturatef(v.z) * 255.0f), a = __float2uint_rn(__saturatef(v.w) * 255.0f);
    out[(size_t)y * w + x] = r | (g << 8) | (b << 16) | (a << 24);
}

#define CHECK(call)                                                               \
    do {                                                                          \
        const cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                                  \
            std::fprintf(stderr, "%s: %s\n", #call, cudaGetErrorString(e_));     \
            return 1;                                                             \
        }                                                                         \
    } while (0)

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: bc_hw format blocks.bin rgba.bin width height\n");
        return 2;
    }
    const int format = std::atoi(argv[1]);
    const unsigned w = (unsigned)std::atoi(argv[4]), h = (unsigned)std::atoi(argv[5]);
    cudaChannelFormatDesc desc;
    size_t block_bytes = 16;
    switch (format) {
        case 1:
            desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsignedBlockCompressed1);
            block_bytes = 8;
            break;
        case 2: desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsignedBlockCompressed2); break;
        case 3: desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsignedBlockCompressed3); break;
        case 4:
            desc = cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindUnsignedBlockCompressed4);
            block_bytes = 8;
            break;
        case 5: desc = cudaCreateChannelDesc(8, 8, 0, 0, cudaChannelFormatKindUnsignedBlockCompressed5); break;
        case 8: desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsignedBlockCompressed7); break;
        case 9: desc = cudaCreateChannelDesc(16, 16, 16, 0, cudaChannelFormatKindUnsignedBlockCompressed6H); break;
        case 10: desc = cudaCreateChannelDesc(16, 16, 16, 0, cudaChannelFormatKindSignedBlockCompressed6H); break;
        default: std::fprintf(stderr, "unknown format %d\n", format); return 2;
    }
    if (w == 0 || h == 0 || w % 4 || h % 4 || w > 4096 || h > 4096) {
        std::fprintf(stderr, "width and height must be multiples of 4 in [4, 4096]\n");
        return 2;
    }
    const size_t row_bytes = (size_t)(w / 4) * block_bytes, rows = h / 4;
    std::vector<unsigned char> blocks(row_bytes * rows);
    FILE* f = std::fopen(argv[2], "rb");
    if (!f || std::fread(blocks.data(), 1, blocks.size(), f) != blocks.size()) {
        std::fprintf(stderr, "cannot read %zu block bytes from %s\n", blocks.size(), argv[2]);
        return 2;
    }
    std::fclose(f);

    cudaArray_t array = nullptr;
    CHECK(cudaMallocArray(&array, &desc, w, h));
    // a block-compressed array is copied as rows of blocks
    CHECK(cudaMemcpy2DToArray(array, 0, 0, blocks.data(), row_bytes, row_bytes, rows, cudaMemcpyHostToDevice));
    cudaResourceDesc res = {};
    res.resType = cudaResourceTypeArray;
    res.res.array.array = array;
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModePoint;
    const bool hdr = format == 9 || format == 10;
    td.readMode = hdr ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
    td.normalizedCoords = 0;
    cudaTextureObject_t tex = 0;
    CHECK(cudaCreateTextureObject(&tex, &res, &td, nullptr));
    const size_t words = (size_t)w * h * (hdr ? 4 : 1);
    unsigned* out = nullptr;
    CHECK(cudaMalloc(&out, words * 4));
    if (hdr)
        k_fetch_float<<<dim3((w + 127) / 128, h), 128>>>(tex, w, h, reinterpret_cast<float4*>(out));
    else
        k_fetch<<<dim3((w + 127) / 128, h), 128>>>(tex, w, h, out);
    CHECK(cudaGetLastError());
    CHECK(cudaDeviceSynchronize());
    std::vector<unsigned> host(words);
    CHECK(cudaMemcpy(host.data(), out, host.size() * 4, cudaMemcpyDeviceToHost));
    CHECK(cudaDestroyTextureObject(tex));
    CHECK(cudaFreeArray(array));
    CHECK(cudaFree(out));
    f = std::fopen(argv[3], "wb");
    if (!f || std::fwrite(host.data(), 4, host.size(), f) != host.size()) {
        std::fprintf(stderr, "cannot write %s\n", argv[3]);
        return 2;
    }
    std::fclose(f);
    return 0;
}
