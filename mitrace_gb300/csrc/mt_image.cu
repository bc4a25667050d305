// mt_image.cu - image output: the RGB8 conversion of RenderBuffer::GetPixelsRGB8
// (src/Tracer/RenderBuffer.cpp:37-58) as a device kernel over the rendered
// image, and dependency-free PNG / Radiance HDR writers for the host copy
// (RenderBuffer::SaveToFilePNG / SaveToFileHDR, RenderBuffer.cpp:60-84).
//
// PNG: 8-bit RGB, filter 0 on every row, zlib stream of stored (uncompressed)
// deflate blocks (RFC 1950/1951), CRC-32 per chunk (RFC 2083).  HDR: the
// Radiance RGBE format (Ward's shared-exponent pixels), new-style scanlines
// whose channels are stored as literal runs (flat scanlines outside the
// widths that format allows).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/mitrace_gpu.h"
#include "mt_internal.h"

namespace mt {
namespace {

// FloatToU8: clamp(v * 255, 0, 255) then truncation to uint8.
__global__ void k_rgb8(const float* __restrict__ rgb, uint64_t n, uint8_t* __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const float v = fminf(fmaxf(__fmul_rn(rgb[i], 255.0f), 0.0f), 255.0f);
        out[i] = static_cast<uint8_t>(v);
    }
}

struct CrcTable {
    uint32_t t[256];
    CrcTable()
    {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t x = i;
            for (int k = 0; k < 8; ++k) x = (x & 1u) ? 0xEDB88320u ^ (x >> 1) : x >> 1;
            t[i] = x;
        }
    }
};

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu)
{
    static const CrcTable table;  // initialised once, thread-safe
    for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c;
}

void put32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back(static_cast<uint8_t>(x >> 24));
    v.push_back(static_cast<uint8_t>(x >> 16));
    v.push_back(static_cast<uint8_t>(x >> 8));
    v.push_back(static_cast<uint8_t>(x));
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& body)
{
    put32(out, static_cast<uint32_t>(body.size()));
    const size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), body.begin(), body.end());
    put32(out, crc32(out.data() + start, out.size() - start) ^ 0xFFFFFFFFu);
}

bool write_file(const char* path, const std::vector<uint8_t>& bytes)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    return std::fclose(f) == 0 && ok;
}

}  // namespace
}  // namespace mt

extern "C" {

mt_status mt_image_rgb8(const float* d_rgb, uint32_t width, uint32_t height, uint8_t* d_rgb8, void* cuda_stream)
{
    if (!d_rgb || !d_rgb8 || !width || !height) return mt::internal_error(MT_ERR_INVALID, "null or empty image");
    const uint64_t n = 3ull * width * height;
    const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((n + 255) / 256, 65535));
    mt::k_rgb8<<<blocks, 256, 0, static_cast<cudaStream_t>(cuda_stream)>>>(d_rgb, n, d_rgb8);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mt::internal_error(MT_ERR_CUDA, cudaGetErrorString(e));
    return MT_OK;
}

mt_status mt_write_png(const char* path, const uint8_t* rgb8, uint32_t width, uint32_t height)
{
    if (!path || !rgb8 || !width || !height) return mt::internal_error(MT_ERR_INVALID, "null or empty image");
    using mt::put32;
    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, width);
    put32(ihdr, height);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit RGB, deflate, filter set 0, no interlace
    mt::chunk(out, "IHDR", ihdr);
    // raw scanlines: filter byte 0 + RGB
    const size_t row = 3ull * width;
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * height);
    for (uint32_t y = 0; y < height; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgb8 + y * row, rgb8 + (y + 1) * row);
    }
    // zlib: header, stored blocks of at most 65535 bytes, Adler-32
    std::vector<uint8_t> z = {0x78, 0x01};
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        z.push_back(off + len >= raw.size() ? 1 : 0);
        z.push_back(static_cast<uint8_t>(len));
        z.push_back(static_cast<uint8_t>(len >> 8));
        z.push_back(static_cast<uint8_t>(~len));
        z.push_back(static_cast<uint8_t>(~len >> 8));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        if (raw.empty()) break;
    }
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(z, (b << 16) | a);
    mt::chunk(out, "IDAT", z);
    mt::chunk(out, "IEND", {});
    if (!mt::write_file(path, out)) return mt::internal_error(MT_ERR_INVALID, std::string("cannot write ") + path);
    return MT_OK;
}

mt_status mt_write_hdr(const char* path, const float* rgb, uint32_t width, uint32_t height)
{
    if (!path || !rgb || !width || !height) return mt::internal_error(MT_ERR_INVALID, "null or empty image");
    const std::string head = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(height) + " +X " +
                             std::to_string(width) + "\n";
    std::vector<uint8_t> out(head.begin(), head.end());
    out.reserve(out.size() + 4ull * width * height + 8ull * height);
    std::vector<uint8_t> line(4ull * width);
    const bool rle = width >= 8 && width < 32768;
    for (uint32_t y = 0; y < height; ++y) {
        for (uint32_t x = 0; x < width; ++x) {
            const float* px = rgb + 3ull * (static_cast<uint64_t>(y) * width + x);
            const float m = std::max(px[0], std::max(px[1], px[2]));
            uint8_t* q = &line[4ull * x];
            if (!(m >= 1e-32f)) {  // also maps NaN to black
                q[0] = q[1] = q[2] = q[3] = 0;
                continue;
            }
            int e = 0;
            const float mant = std::frexp(m, &e);  // m = mant * 2^e, mant in [0.5, 1)
            const float sc = mant * 256.0f / m;
            for (int c = 0; c < 3; ++c) q[c] = static_cast<uint8_t>(std::max(0.0f, px[c]) * sc);
            q[3] = static_cast<uint8_t>(e + 128);
        }
        if (!rle) {
            out.insert(out.end(), line.begin(), line.end());
            continue;
        }
        // new-style scanline: marker, then each channel as literal runs of <= 128
        out.insert(out.end(), {2, 2, static_cast<uint8_t>(width >> 8), static_cast<uint8_t>(width & 0xFF)});
        for (int c = 0; c < 4; ++c)
            for (uint32_t x = 0; x < width; x += 128) {
                const uint32_t n = std::min<uint32_t>(128, width - x);
                out.push_back(static_cast<uint8_t>(n));
                for (uint32_t k = 0; k < n; ++k) out.push_back(line[4ull * (x + k) + c]);
            }
    }
    if (!mt::write_file(path, out)) return mt::internal_error(MT_ERR_INVALID, std::string("cannot write ") + path);
    return MT_OK;
}

}  // extern "C"
