// video_decode.hpp -- uncompressed video containers for smip-cli: SER and AVI.
//
// The reference reads video through OpenCV's VideoCapture (FrameExtractor,
// src/videoio.cpp:13-52), which hands every frame over as an 8-bit BGR
// image; Mat2Array then picks one channel of it (include/videoio.h:71-98).
// Speckle data is usually recorded as SER (the astronomy capture format) or
// as uncompressed AVI, and often with 16-bit samples, which that path reads
// as zeros.  These readers deliver the frames in the layout the rest of
// smip-cli takes: [rows][cols] per frame for one-channel data and
// [rows][cols][3] in B, G, R order for colour data, top row first, 1 or 2
// bytes per sample in host byte order.  Frames stay in the file and are read
// one at a time (read_frame), so stacks larger than host memory work.
//
// SER (Lucam Recorder format, version 3): a 178-byte little-endian header
//   0 "LUCAM-RECORDER", 14 LuID, 18 ColorID, 22 LittleEndian, 26 ImageWidth,
//   30 ImageHeight, 34 PixelDepthPerPlane, 38 FrameCount, 42-161 observer,
//   instrument and telescope strings, 162/170 two 64-bit time stamps,
// then FrameCount frames of width x height x planes samples, 1 byte each for
// a pixel depth of 1-8 bits and 2 bytes for 9-16.  ColorID 0 is mono; 8-19
// are raw Bayer mosaics, delivered as one channel (the mosaic itself); 100
// (RGB) and 101 (BGR) have three planes per pixel and are delivered as B, G,
// R.  LittleEndian is read as the format defines it: non-zero means 16-bit
// samples are little-endian, zero means big-endian.  A trailer of frame time
// stamps after the frames is ignored.
//
// AVI (RIFF "AVI ", and the "AVIX" extensions of OpenDML files for more than
// 1 GB): the first video stream's BITMAPINFOHEADER decides the sample layout,
// and its frames are the "##db" / "##dc" chunks of every "movi" list, in file
// order (no index is needed).  Supported: BI_RGB with 24 bits (BGR) or 32
// bits (BGRX, the fourth byte dropped), rows padded to 4 bytes, bottom-up for
// a positive height and top-down for a negative one; BI_RGB with 8 bits and
// a colour table (delivered as B, G, R through the table, as VideoCapture
// does); "Y800" / "Y8  " / "GREY" 8-bit and "Y16 " 16-bit little-endian
// gray, top row first, unpadded.  A chunk of size zero (a dropped frame)
// repeats the previous frame, as players show it.  Compressed streams are
// refused.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace smipcli {

class VideoSource {
public:
    std::size_t width = 0, height = 0, channels = 1, count = 0;
    int esize = 1; // bytes per sample (1 or 2)

    // Frame idx into out (height * width * channels * esize bytes).
    void read_frame(std::size_t idx, void* out) const
    {
        if (idx >= count)
            throw std::out_of_range("video frame index out of range");
        const std::size_t fbytes = height * width * channels * (std::size_t)esize;
        raw_.resize(in_bytes_);
        // a dropped AVI frame (chunk of size zero) repeats the last real one
        std::size_t k = idx;
        while (k > 0 && offs_[k] < 0)
            --k;
        if (offs_[k] < 0) {
            std::memset(out, 0, fbytes);
            return;
        }
        if (std::fseek(f_.get(), offs_[k], SEEK_SET) != 0 || std::fread(raw_.data(), 1, in_bytes_, f_.get()) != in_bytes_)
            throw std::runtime_error("error reading frame " + std::to_string(idx));
        convert(raw_.data(), static_cast<std::uint8_t*>(out));
    }

    static bool is_ser(const std::string& path) { return magic(path, "LUCAM-RECORDER", 14); }
    static bool is_avi(const std::string& path)
    {
        std::uint8_t h[12];
        return head(path, h, 12) && std::memcmp(h, "RIFF", 4) == 0 && std::memcmp(h + 8, "AVI ", 4) == 0;
    }

    static VideoSource open_ser(const std::string& path)
    {
        VideoSource v;
        v.open_file(path);
        std::uint8_t h[178];
        if (std::fread(h, 1, 178, v.f_.get()) != 178 || std::memcmp(h, "LUCAM-RECORDER", 14) != 0)
            throw std::runtime_error(path + ": not a SER file");
        const std::int32_t color = le32s(h + 18), little = le32s(h + 22), w = le32s(h + 26), hh = le32s(h + 30),
                           depth = le32s(h + 34), n = le32s(h + 38);
        if (w <= 0 || hh <= 0 || n < 0 || depth < 1 || depth > 16)
            throw std::runtime_error(path + ": invalid SER header");
        v.width = (std::size_t)w;
        v.height = (std::size_t)hh;
        v.esize = depth <= 8 ? 1 : 2;
        v.swap16_ = v.esize == 2 && little == 0;
        if (color == 100 || color == 101) {
            v.channels = 3;
            v.rgb_ = color == 100; // RGB planes are delivered as B, G, R
        } else if (color == 0 || (color >= 8 && color <= 19)) {
            v.channels = 1;
        } else {
            throw std::runtime_error(path + ": unknown SER ColorID " + std::to_string(color));
        }
        v.in_bytes_ = v.width * v.height * v.channels * (std::size_t)v.esize;
        const long fsz = file_size(v.f_.get());
        const long have = v.in_bytes_ ? (fsz - 178) / (long)v.in_bytes_ : 0;
        v.count = (std::size_t)std::min<long>(n, have); // a truncated recording keeps its whole frames
        v.offs_.resize(v.count);
        for (std::size_t k = 0; k < v.count; ++k)
            v.offs_[k] = 178 + (long)(k * v.in_bytes_);
        v.kind_ = Kind::Plain;
        return v;
    }

    static VideoSource open_avi(const std::string& path)
    {
        VideoSource v;
        v.open_file(path);
        FILE* f = v.f_.get();
        const long fsz = file_size(f);
        long pos = 0;
        int vstream = -1;
        bool have_fmt = false;
        std::int32_t bw = 0, bh = 0;
        std::uint16_t bits = 0;
        std::uint32_t comp = 0;
        std::vector<std::uint8_t> pal;
        // top level: RIFF AVI / RIFF AVIX chunks
        while (pos + 12 <= fsz) {
            std::uint8_t c[12];
            if (!read_at(f, pos, c, 12))
                break;
            const std::uint32_t sz = le32(c + 4);
            if (std::memcmp(c, "RIFF", 4) != 0)
                break;
            const long end = std::min<long>(fsz, pos + 8 + (long)sz);
            walk(f, pos + 12, end, [&](const std::uint8_t* id, long body, std::uint32_t len, const char* list) {
                if (std::memcmp(id, "strh", 4) == 0 && len >= 8) {
                    std::uint8_t t[4];
                    read_at(f, body, t, 4);
                    ++v.nstreams_;
                    if (vstream < 0 && std::memcmp(t, "vids", 4) == 0)
                        vstream = v.nstreams_ - 1;
                } else if (std::memcmp(id, "strf", 4) == 0 && vstream == v.nstreams_ - 1 && !have_fmt && len >= 40) {
                    std::vector<std::uint8_t> b(len);
                    read_at(f, body, b.data(), len);
                    bw = le32s(b.data() + 4);
                    bh = le32s(b.data() + 8);
                    bits = le16(b.data() + 14);
                    comp = le32(b.data() + 16);
                    const std::uint32_t hdr = le32(b.data());
                    if (bits == 8 && comp == 0 && len > hdr)
                        pal.assign(b.begin() + hdr, b.end());
                    have_fmt = true;
                } else if (vstream >= 0 && list && std::memcmp(list, "movi", 4) == 0 && is_frame(id, vstream)) {
                    v.offs_.push_back(len ? body : -1);
                    v.lens_.push_back(len);
                }
            });
            pos += 8 + (long)sz + (sz & 1);
        }
        if (!have_fmt || bw <= 0 || bh == 0)
            throw std::runtime_error(path + ": no video stream format in the AVI file");
        v.width = (std::size_t)bw;
        v.height = (std::size_t)(bh < 0 ? -bh : bh);
        v.bottom_up_ = bh > 0;
        const std::uint32_t Y800 = fourcc("Y800"), Y8 = fourcc("Y8  "), GREY = fourcc("GREY"), Y16 = fourcc("Y16 ");
        if (comp == 0 && (bits == 24 || bits == 32)) {
            v.kind_ = Kind::Bgr;
            v.channels = 3;
            v.in_stride_ = (v.width * (bits / 8) + 3) / 4 * 4;
            v.in_pix_ = bits / 8;
        } else if (comp == 0 && bits == 8) {
            if (pal.size() < 4)
                throw std::runtime_error(path + ": 8-bit AVI without a colour table");
            v.kind_ = Kind::Palette;
            v.channels = 3;
            v.in_stride_ = (v.width + 3) / 4 * 4;
            v.pal_ = pal;
        } else if ((comp == Y800 || comp == Y8 || comp == GREY) && bits == 8) {
            v.kind_ = Kind::Plain;
            v.bottom_up_ = false;
            v.in_stride_ = v.width;
        } else if (comp == Y16 && bits == 16) {
            v.kind_ = Kind::Plain;
            v.bottom_up_ = false;
            v.esize = 2;
            v.in_stride_ = v.width * 2;
        } else {
            throw std::runtime_error(path + ": unsupported AVI video format (compressed, or " + std::to_string(bits)
                                     + "-bit); uncompressed 8/24/32-bit BI_RGB, Y800/GREY or Y16 only");
        }
        v.in_bytes_ = v.kind_ == Kind::Plain && v.in_stride_ == v.width * v.esize ? v.width * v.height * v.esize
                                                                                   : v.in_stride_ * v.height;
        for (std::size_t k = 0; k < v.offs_.size(); ++k)
            if (v.offs_[k] >= 0 && v.lens_[k] < v.in_bytes_)
                throw std::runtime_error(path + ": frame " + std::to_string(k) + " is shorter than the format says");
        v.count = v.offs_.size();
        return v;
    }

private:
    enum class Kind { Plain, Bgr, Palette };
    struct Closer {
        void operator()(FILE* f) const
        {
            if (f)
                std::fclose(f);
        }
    };
    std::shared_ptr<FILE> f_;
    Kind kind_ = Kind::Plain;
    std::vector<long> offs_;            // per frame: file offset of its samples, -1 for a dropped frame
    std::vector<std::uint32_t> lens_;
    std::size_t in_bytes_ = 0;          // bytes of one stored frame
    std::size_t in_stride_ = 0;         // bytes of one stored row (AVI)
    std::size_t in_pix_ = 3;            // bytes per stored pixel (BGR kinds)
    bool bottom_up_ = false, swap16_ = false, rgb_ = false;
    std::vector<std::uint8_t> pal_;     // RGBQUAD colour table (B, G, R, reserved)
    int nstreams_ = 0;
    mutable std::vector<std::uint8_t> raw_;

    void open_file(const std::string& path)
    {
        FILE* f = std::fopen(path.c_str(), "rb");
        if (!f)
            throw std::runtime_error("file open error: " + path);
        f_ = std::shared_ptr<FILE>(f, Closer());
    }

    void convert(const std::uint8_t* in, std::uint8_t* out) const
    {
        const std::size_t W = width, H = height;
        if (kind_ == Kind::Plain) {
            const std::size_t row = W * channels * (std::size_t)esize;
            const std::size_t stride = in_stride_ ? in_stride_ : row;
            for (std::size_t y = 0; y < H; ++y) {
                const std::uint8_t* src = in + (bottom_up_ ? H - 1 - y : y) * stride;
                std::uint8_t* dst = out + y * row;
                if (esize == 2) {
                    for (std::size_t q = 0; q < W * channels; ++q) {
                        const std::uint16_t s = swap16_ ? (std::uint16_t)((src[2 * q] << 8) | src[2 * q + 1])
                                                        : (std::uint16_t)(src[2 * q] | (src[2 * q + 1] << 8));
                        std::memcpy(dst + 2 * q, &s, 2);
                    }
                } else {
                    std::memcpy(dst, src, row);
                }
                if (rgb_) // R, G, B planes -> B, G, R
                    for (std::size_t x = 0; x < W; ++x) {
                        std::uint8_t* p = dst + x * 3 * esize;
                        for (int b = 0; b < esize; ++b)
                            std::swap(p[b], p[2 * esize + b]);
                    }
            }
        } else if (kind_ == Kind::Bgr) {
            for (std::size_t y = 0; y < H; ++y) {
                const std::uint8_t* src = in + (bottom_up_ ? H - 1 - y : y) * in_stride_;
                std::uint8_t* dst = out + y * W * 3;
                for (std::size_t x = 0; x < W; ++x)
                    std::memcpy(dst + 3 * x, src + in_pix_ * x, 3);
            }
        } else {
            const std::size_t npal = pal_.size() / 4;
            for (std::size_t y = 0; y < H; ++y) {
                const std::uint8_t* src = in + (bottom_up_ ? H - 1 - y : y) * in_stride_;
                std::uint8_t* dst = out + y * W * 3;
                for (std::size_t x = 0; x < W; ++x) {
                    const std::size_t i = src[x] < npal ? src[x] : 0;
                    std::memcpy(dst + 3 * x, pal_.data() + 4 * i, 3);
                }
            }
        }
    }

    static std::uint32_t fourcc(const char* s) { return le32(reinterpret_cast<const std::uint8_t*>(s)); }
    static std::uint16_t le16(const std::uint8_t* p) { return (std::uint16_t)(p[0] | (p[1] << 8)); }
    static std::uint32_t le32(const std::uint8_t* p)
    {
        return (std::uint32_t)p[0] | ((std::uint32_t)p[1] << 8) | ((std::uint32_t)p[2] << 16) | ((std::uint32_t)p[3] << 24);
    }
    static std::int32_t le32s(const std::uint8_t* p) { return (std::int32_t)le32(p); }

    static bool is_frame(const std::uint8_t* id, int stream)
    {
        const int d0 = id[0] - '0', d1 = id[1] - '0';
        if (d0 < 0 || d0 > 9 || d1 < 0 || d1 > 9 || d0 * 10 + d1 != stream)
            return false;
        return (id[2] == 'd' && (id[3] == 'b' || id[3] == 'c'));
    }

    static bool read_at(FILE* f, long pos, void* buf, std::size_t n)
    {
        return std::fseek(f, pos, SEEK_SET) == 0 && std::fread(buf, 1, n, f) == n;
    }

    static long file_size(FILE* f)
    {
        std::fseek(f, 0, SEEK_END);
        return std::ftell(f);
    }

    static bool head(const std::string& path, std::uint8_t* h, std::size_t n)
    {
        FILE* f = std::fopen(path.c_str(), "rb");
        if (!f)
            return false;
        const bool ok = std::fread(h, 1, n, f) == n;
        std::fclose(f);
        return ok;
    }

    static bool magic(const std::string& path, const char* m, std::size_t n)
    {
        std::vector<std::uint8_t> h(n);
        return head(path, h.data(), n) && std::memcmp(h.data(), m, n) == 0;
    }

    // Visits the chunks in [pos, end): fn(id, body offset, body length, enclosing list type or null),
    // descending into LIST chunks (depth-first, in file order).
    template <class F>
    static void walk(FILE* f, long pos, long end, F&& fn, const char* list = nullptr, int depth = 0)
    {
        while (pos + 8 <= end) {
            std::uint8_t c[12];
            if (!read_at(f, pos, c, 8))
                return;
            const std::uint32_t len = le32(c + 4);
            const long body = pos + 8;
            if (body + (long)len > end)
                return; // truncated file: keep what came before
            if (std::memcmp(c, "LIST", 4) == 0 && len >= 4 && depth < 8) {
                char type[4];
                if (!read_at(f, body, type, 4))
                    return;
                const char* inner = std::memcmp(type, "rec ", 4) == 0 && list ? list : type;
                walk(f, body + 4, body + (long)len, fn, inner, depth + 1);
            } else {
                fn(c, body, len, list);
            }
            pos = body + (long)len + (len & 1);
        }
    }
};

} // namespace smipcli
