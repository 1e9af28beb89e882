// gif_decode.hpp -- GIF87a / GIF89a frame decoder for smip-cli.
//
// The reference reads video and animated GIF files through OpenCV's
// VideoCapture (FrameExtractor, src/videoio.cpp:13-52), which delivers every
// frame as the full logical screen in 8-bit BGR order; Mat2Array then picks
// one channel of it (include/videoio.h:71-98).  This decoder produces the same
// layout: frames [count][height][width][3], channels B, G, R.
//
// Every frame is drawn onto the logical screen (its sub-rectangle, its local
// or the global colour table, interlaced rows, the transparent index of its
// graphic control extension); the disposal method of a frame (keep, restore
// to background, restore to previous) is applied before the next one is
// drawn.  The canvas starts black.  Image data is LZW (variable code width
// from the minimum code size + 1 up to 12 bits, clear and end codes).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace smipcli {

struct GifFrames {
    std::size_t width = 0, height = 0, count = 0;
    std::vector<std::uint8_t> bgr; // [count][height][width][3]
};

namespace gifdetail {

inline std::uint16_t le16(const std::uint8_t* p) { return (std::uint16_t)(p[0] | (p[1] << 8)); }

// LZW decode of one image's data sub-blocks into npix colour indices.
inline std::vector<std::uint8_t> lzw_decode(const std::vector<std::uint8_t>& data, int min_code, std::size_t npix)
{
    if (min_code < 2 || min_code > 11)
        throw std::runtime_error("GIF: invalid LZW minimum code size");
    const int clear = 1 << min_code, eoi = clear + 1;
    std::vector<std::uint16_t> prefix(4096);
    std::vector<std::uint8_t> suffix(4096), stack(4097);
    std::vector<std::uint8_t> out;
    out.reserve(npix);
    for (int i = 0; i < clear; ++i) {
        prefix[i] = 0xffff;
        suffix[i] = (std::uint8_t)i;
    }
    int width = min_code + 1, next = eoi + 1, prev = -1;
    std::uint8_t first = 0;
    std::uint32_t bits = 0;
    int nbits = 0;
    std::size_t pos = 0;
    while (out.size() < npix) {
        while (nbits < width && pos < data.size()) {
            bits |= (std::uint32_t)data[pos++] << nbits;
            nbits += 8;
        }
        if (nbits < width)
            break; // data ended early: the rest of the image stays at index 0
        const int code = (int)(bits & ((1u << width) - 1));
        bits >>= width;
        nbits -= width;
        if (code == clear) {
            width = min_code + 1;
            next = eoi + 1;
            prev = -1;
            continue;
        }
        if (code == eoi)
            break;
        int cur = code, sp = 0;
        if (prev < 0) {
            if (code >= clear)
                throw std::runtime_error("GIF: corrupt LZW data");
            out.push_back((std::uint8_t)code);
            first = (std::uint8_t)code;
            prev = code;
            continue;
        }
        if (code > next)
            throw std::runtime_error("GIF: corrupt LZW data");
        if (code == next) { // the KwKwK case
            stack[sp++] = first;
            cur = prev;
        }
        while (cur >= clear) {
            stack[sp++] = suffix[cur];
            cur = prefix[cur];
        }
        stack[sp++] = (std::uint8_t)cur;
        first = (std::uint8_t)cur;
        while (sp > 0 && out.size() < npix)
            out.push_back(stack[--sp]);
        if (next < 4096) {
            prefix[next] = (std::uint16_t)prev;
            suffix[next] = first;
            ++next;
            if (next == (1 << width) && width < 12)
                ++width;
        }
        prev = code;
    }
    out.resize(npix, 0);
    return out;
}

} // namespace gifdetail

inline bool is_gif(const std::string& path)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f)
        return false;
    char m[4] = {};
    const bool ok = std::fread(m, 1, 4, f) == 4 && m[0] == 'G' && m[1] == 'I' && m[2] == 'F' && m[3] == '8';
    std::fclose(f);
    return ok;
}

inline GifFrames read_gif(const std::string& path, std::size_t max_frames = (std::size_t)-1)
{
    using namespace gifdetail;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f)
        throw std::runtime_error("file open error: " + path);
    std::vector<std::uint8_t> d;
    std::uint8_t buf[65536];
    std::size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0)
        d.insert(d.end(), buf, buf + n);
    std::fclose(f);
    auto need = [&](std::size_t p, std::size_t k) {
        if (p + k > d.size())
            throw std::runtime_error(path + ": truncated GIF");
    };
    need(0, 13);
    if (d[0] != 'G' || d[1] != 'I' || d[2] != 'F')
        throw std::runtime_error(path + ": not a GIF file");
    GifFrames g;
    g.width = le16(&d[6]);
    g.height = le16(&d[8]);
    const std::uint8_t lsd = d[10];
    const std::uint8_t bg_index = d[11];
    std::size_t p = 13;
    std::vector<std::uint8_t> gct;
    if (lsd & 0x80) {
        const std::size_t sz = 3u << ((lsd & 7) + 1);
        need(p, sz);
        gct.assign(d.begin() + p, d.begin() + p + sz);
        p += sz;
    }
    const std::size_t W = g.width, H = g.height;
    std::vector<std::uint8_t> canvas(W * H * 3, 0), saved;
    int transparent = -1, disposal = 0;
    auto sub_blocks = [&](std::vector<std::uint8_t>* out) {
        for (;;) {
            need(p, 1);
            const std::size_t k = d[p++];
            if (k == 0)
                return;
            need(p, k);
            if (out)
                out->insert(out->end(), d.begin() + p, d.begin() + p + k);
            p += k;
        }
    };
    while (p < d.size() && g.count < max_frames) {
        const std::uint8_t b = d[p++];
        if (b == 0x3B) // trailer
            break;
        if (b == 0x21) { // extension
            need(p, 1);
            const std::uint8_t label = d[p++];
            if (label == 0xF9) { // graphic control extension
                std::vector<std::uint8_t> gce;
                sub_blocks(&gce);
                if (gce.size() >= 4) {
                    disposal = (gce[0] >> 2) & 7;
                    transparent = (gce[0] & 1) ? gce[3] : -1;
                }
            } else {
                sub_blocks(nullptr);
            }
            continue;
        }
        if (b != 0x2C)
            throw std::runtime_error(path + ": unexpected GIF block");
        need(p, 9);
        const std::size_t fl = le16(&d[p]), ft = le16(&d[p + 2]), fw = le16(&d[p + 4]), fh = le16(&d[p + 6]);
        const std::uint8_t idp = d[p + 8];
        p += 9;
        std::vector<std::uint8_t> lct;
        if (idp & 0x80) {
            const std::size_t sz = 3u << ((idp & 7) + 1);
            need(p, sz);
            lct.assign(d.begin() + p, d.begin() + p + sz);
            p += sz;
        }
        const std::vector<std::uint8_t>& ct = lct.empty() ? gct : lct;
        need(p, 1);
        const int min_code = d[p++];
        std::vector<std::uint8_t> data;
        sub_blocks(&data);
        const std::vector<std::uint8_t> idx = lzw_decode(data, min_code, fw * fh);
        if (disposal == 3)
            saved = canvas;
        // rows of an interlaced image come in passes 0,8,16..; 4,12..; 2,6..; 1,3..
        std::vector<std::size_t> rowmap(fh);
        if (idp & 0x40) {
            std::size_t r = 0;
            const std::size_t start[4] = { 0, 4, 2, 1 }, step[4] = { 8, 8, 4, 2 };
            for (int pass = 0; pass < 4; ++pass)
                for (std::size_t y = start[pass]; y < fh; y += step[pass])
                    rowmap[r++] = y;
        } else {
            for (std::size_t y = 0; y < fh; ++y)
                rowmap[y] = y;
        }
        for (std::size_t r = 0; r < fh; ++r) {
            const std::size_t y = ft + rowmap[r];
            if (y >= H)
                continue;
            for (std::size_t x = 0; x < fw; ++x) {
                const std::size_t cx = fl + x;
                const int c = idx[r * fw + x];
                if (cx >= W || c == transparent || 3 * (std::size_t)c + 2 >= ct.size())
                    continue;
                std::uint8_t* px = &canvas[3 * (y * W + cx)];
                px[0] = ct[3 * c + 2]; // B
                px[1] = ct[3 * c + 1]; // G
                px[2] = ct[3 * c];     // R
            }
        }
        g.bgr.insert(g.bgr.end(), canvas.begin(), canvas.end());
        ++g.count;
        if (disposal == 2) { // restore the frame's rectangle to the background colour
            std::uint8_t bgc[3] = { 0, 0, 0 };
            if (transparent < 0 && 3 * (std::size_t)bg_index + 2 < gct.size()) {
                bgc[0] = gct[3 * bg_index + 2];
                bgc[1] = gct[3 * bg_index + 1];
                bgc[2] = gct[3 * bg_index];
            }
            for (std::size_t y = ft; y < ft + fh && y < H; ++y)
                for (std::size_t x = fl; x < fl + fw && x < W; ++x)
                    for (int k = 0; k < 3; ++k)
                        canvas[3 * (y * W + x) + k] = bgc[k];
        } else if (disposal == 3) {
            canvas = saved;
        }
        transparent = -1;
        disposal = 0;
    }
    return g;
}

} // namespace smipcli
