// png.cpp -- minimal PNG writer for the headless renderer: 8-bit RGB, one
// zlib stream of stored (uncompressed) deflate blocks, CRC-32 per chunk.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace sonar {
namespace {

uint32_t crc_table[256];
bool crc_ready = false;

uint32_t crc32(const unsigned char *p, size_t n, uint32_t c = 0xFFFFFFFFu)
{
    if (!crc_ready) {
        for (uint32_t k = 0; k < 256; k++) {
            uint32_t v = k;
            for (int b = 0; b < 8; b++) v = (v & 1u) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            crc_table[k] = v;
        }
        crc_ready = true;
    }
    for (size_t i = 0; i < n; i++) c = crc_table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c;
}

void put32(std::vector<unsigned char> &o, uint32_t v)
{
    o.push_back((unsigned char)(v >> 24));
    o.push_back((unsigned char)(v >> 16));
    o.push_back((unsigned char)(v >> 8));
    o.push_back((unsigned char)v);
}

void chunk(std::vector<unsigned char> &o, const char *type, const std::vector<unsigned char> &data)
{
    put32(o, (uint32_t)data.size());
    const size_t start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put32(o, crc32(o.data() + start, o.size() - start) ^ 0xFFFFFFFFu);
}

}  // namespace

// rgb: height rows of width x 3 bytes, top row first.  Returns false on an I/O error.
bool write_png(const std::string &path, int width, int height, const unsigned char *rgb)
{
    std::vector<unsigned char> raw;
    raw.reserve((size_t)height * ((size_t)width * 3 + 1));
    for (int y = 0; y < height; y++) {
        raw.push_back(0);  // filter: none
        raw.insert(raw.end(), rgb + (size_t)y * width * 3, rgb + (size_t)(y + 1) * width * 3);
    }
    std::vector<unsigned char> z = {0x78, 0x01};  // zlib header, no compression
    uint32_t a = 1, b = 0;
    for (unsigned char c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        z.push_back(off + len >= raw.size() ? 1 : 0);  // final block flag, stored
        z.push_back((unsigned char)(len & 0xFF));
        z.push_back((unsigned char)(len >> 8));
        z.push_back((unsigned char)(~len & 0xFF));
        z.push_back((unsigned char)((~len >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        if (raw.empty()) break;
    }
    put32(z, (b << 16) | a);
    std::vector<unsigned char> o = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<unsigned char> ihdr;
    put32(ihdr, (uint32_t)width);
    put32(ihdr, (uint32_t)height);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit, RGB, deflate, no filter, no interlace
    chunk(o, "IHDR", ihdr);
    chunk(o, "IDAT", z);
    chunk(o, "IEND", {});
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(o.data(), 1, o.size(), f) == o.size();
    return fclose(f) == 0 && ok;
}

}  // namespace sonar
