// image_io.cpp - writing a rendered film to a file (pbrtgpu_write_image).
//
// Film::write_image (src/camera/film.rs:316-354) hands the final RGB to
// write_img (film.rs:15-33), which stores 8-bit channels
//     byte = (255 * p^(1/2.2) + 0.5) clamped to [0, 255], truncated
// through the `image` crate, the format chosen by the file extension.  Here
// the format also follows the extension: .png and .ppm get those 8-bit
// values (PNG written with stored - uncompressed - deflate blocks, so no
// compression library is needed); .pfm and .exr keep the linear float RGB.  The
// reference's own write_image writes into a buffer of the wrong size and
// overwrites the colour with the splat; the RGB given here is the intended
// value (film_pixel's output).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"

namespace pbrt {
int set_error(int status, const std::string& msg);
}
using pbrt::set_error;

namespace {

// film.rs:22-24 with Rust's f32 powf, `as u8` saturating
uint8_t to_byte(float p) {
    float v = 255.0f * std::pow(p, 1.0f / 2.2f) + 0.5f;
    if (!(v >= 0.0f)) return 0;  // also NaN, as Rust's clamp-then-cast gives 0 for NaN
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}

struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1u) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            t[i] = v;
        }
    }
};

// CRC-32 of the PNG chunks (ISO 3309 polynomial, reflected)
uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu) {
    static const CrcTable table;  // initialised once, thread-safe
    for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    return c;
}

void put32(std::vector<uint8_t>& o, uint32_t v) {
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

void chunk(std::vector<uint8_t>& o, const char* type, const std::vector<uint8_t>& data) {
    put32(o, (uint32_t)data.size());
    size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put32(o, crc32(o.data() + start, o.size() - start) ^ 0xffffffffu);
}

// PNG (ISO/IEC 15948): 8-bit RGB, filter 0 on every row, zlib stream of
// stored deflate blocks (RFC 1950/1951) with its Adler-32.
std::vector<uint8_t> encode_png(const std::vector<uint8_t>& rgb8, uint32_t w, uint32_t h) {
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (3 * (size_t)w + 1));
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgb8.begin() + (size_t)y * 3 * w, rgb8.begin() + (size_t)(y + 1) * 3 * w);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(z, (b << 16) | a);
    std::vector<uint8_t> o = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, w);
    put32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit, RGB, deflate, filter 0, no interlace
    chunk(o, "IHDR", ihdr);
    chunk(o, "IDAT", z);
    chunk(o, "IEND", {});
    return o;
}

void le32(std::vector<uint8_t>& o, uint32_t v) {
    for (int k = 0; k < 4; ++k) o.push_back((uint8_t)(v >> (8 * k)));
}
void le64(std::vector<uint8_t>& o, uint64_t v) {
    for (int k = 0; k < 8; ++k) o.push_back((uint8_t)(v >> (8 * k)));
}
void lef32(std::vector<uint8_t>& o, float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    le32(o, b);
}
// one header attribute: name, type name, byte size, value
void exr_attr(std::vector<uint8_t>& o, const char* name, const char* type, const std::vector<uint8_t>& value) {
    o.insert(o.end(), name, name + std::strlen(name) + 1);
    o.insert(o.end(), type, type + std::strlen(type) + 1);
    le32(o, (uint32_t)value.size());
    o.insert(o.end(), value.begin(), value.end());
}

// OpenEXR (the published file layout, version 2): a single-part scanline
// file, no compression, one scanline per block, channels B, G, R (sorted by
// name, as the format requires) of 32-bit float, linear values as rendered.
std::vector<uint8_t> encode_exr(const float* rgb, uint32_t w, uint32_t h) {
    std::vector<uint8_t> o = {0x76, 0x2f, 0x31, 0x01, 2, 0, 0, 0};  // magic, version 2 (single-part scanline)
    std::vector<uint8_t> ch;
    for (const char* name : {"B", "G", "R"}) {
        ch.insert(ch.end(), name, name + 2);
        le32(ch, 2);                        // pixel type FLOAT
        ch.insert(ch.end(), {0, 0, 0, 0});  // pLinear, reserved
        le32(ch, 1);                        // x sampling
        le32(ch, 1);                        // y sampling
    }
    ch.push_back(0);
    exr_attr(o, "channels", "chlist", ch);
    exr_attr(o, "compression", "compression", {0});  // NO_COMPRESSION
    std::vector<uint8_t> box;
    le32(box, 0);
    le32(box, 0);
    le32(box, w - 1);
    le32(box, h - 1);
    exr_attr(o, "dataWindow", "box2i", box);
    exr_attr(o, "displayWindow", "box2i", box);
    exr_attr(o, "lineOrder", "lineOrder", {0});  // INCREASING_Y
    std::vector<uint8_t> one;
    lef32(one, 1.0f);
    exr_attr(o, "pixelAspectRatio", "float", one);
    std::vector<uint8_t> centre;
    lef32(centre, 0.0f);
    lef32(centre, 0.0f);
    exr_attr(o, "screenWindowCenter", "v2f", centre);
    exr_attr(o, "screenWindowWidth", "float", one);
    o.push_back(0);  // end of header
    const uint64_t block = 8 + (uint64_t)w * 3 * 4;  // y, byte count, B row, G row, R row
    const uint64_t first = o.size() + 8ull * h;
    for (uint32_t y = 0; y < h; ++y) le64(o, first + (uint64_t)y * block);
    for (uint32_t y = 0; y < h; ++y) {
        le32(o, y);
        le32(o, w * 3 * 4);
        const float* row = rgb + (size_t)y * w * 3;
        for (int c : {2, 1, 0})
            for (uint32_t x = 0; x < w; ++x) lef32(o, row[3 * (size_t)x + c]);
    }
    return o;
}

bool ends_with(const std::string& s, const char* suf) {
    const size_t n = std::strlen(suf);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)s[s.size() - n + i]) != suf[i]) return false;
    return true;
}

}  // namespace

extern "C" {

int pbrtgpu_image_bytes(const float* rgb, uint32_t width, uint32_t height, uint8_t* out) {
    if (!rgb || !out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    const size_t n = (size_t)width * height * 3;
    for (size_t i = 0; i < n; ++i) out[i] = to_byte(rgb[i]);
    return PBRT_OK;
}

int pbrtgpu_write_image(const float* rgb, uint32_t width, uint32_t height, const char* path) {
    if (!rgb || !path) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width == 0 || height == 0) return set_error(PBRT_ERR_INVALID_ARGUMENT, "empty image");
    const std::string p(path);
    std::vector<uint8_t> file;
    const size_t n = (size_t)width * height * 3;
    if (ends_with(p, ".exr")) {
        file = encode_exr(rgb, width, height);
    } else if (ends_with(p, ".pfm")) {
        // Portable float map: little-endian (scale -1), rows bottom to top
        std::string hdr = "PF\n" + std::to_string(width) + " " + std::to_string(height) + "\n-1.0\n";
        file.assign(hdr.begin(), hdr.end());
        for (uint32_t y = height; y-- > 0;) {
            const uint8_t* row = reinterpret_cast<const uint8_t*>(rgb + (size_t)y * width * 3);
            for (size_t i = 0; i < (size_t)width * 3; ++i) {
                uint32_t bits;
                std::memcpy(&bits, row + 4 * i, 4);
                for (int k = 0; k < 4; ++k) file.push_back((uint8_t)(bits >> (8 * k)));
            }
        }
    } else {
        std::vector<uint8_t> rgb8(n);
        pbrtgpu_image_bytes(rgb, width, height, rgb8.data());
        if (ends_with(p, ".png")) {
            file = encode_png(rgb8, width, height);
        } else if (ends_with(p, ".ppm")) {
            std::string hdr = "P6\n" + std::to_string(width) + " " + std::to_string(height) + "\n255\n";
            file.assign(hdr.begin(), hdr.end());
            file.insert(file.end(), rgb8.begin(), rgb8.end());
        } else {
            return set_error(PBRT_ERR_UNSUPPORTED, "image format: use .png, .ppm, .pfm or .exr");
        }
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(PBRT_ERR_INVALID_ARGUMENT, "cannot open " + p + " for writing");
    const size_t wrote = std::fwrite(file.data(), 1, file.size(), f);
    const bool ok = std::fclose(f) == 0 && wrote == file.size();
    return ok ? PBRT_OK : set_error(PBRT_ERR_INVALID_ARGUMENT, "short write to " + p);
}

}  // extern "C"
