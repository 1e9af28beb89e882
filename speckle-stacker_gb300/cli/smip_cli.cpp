// smip-cli -- GB300 speckle-masking reconstruction with the reference's
// command line (smip-cli/main.cpp:41-67, 83-207).
//
//   smip-cli [-n N] [-r idx] [-p R] [-b d] [-c r|g|b|i] [-k l:t] [-s w:h] [-v]
//            [--calcsum|--no-calcsum] [--specklemasking|--no-specklemasking]
//            [--version] [-h] <source>
//
// Same flags, defaults and outputs as the reference: at most -n frames, depth
// -b (default 20), reco radius -p (default 2 x the default depth = 40),
// bispectrum.dat, then sum_image, phases, phasecons, powerspec and reco_image
// as 16-bit PNG (gray and false colour) in the working directory.  Like the
// reference, -r, -k, -s, --no-calcsum and --no-specklemasking are parsed and
// have no effect (main.cpp:84-90, 136-167 never use them).
//
// --rings (not a reference flag) selects the ring-parallel phase recovery.
//
// --apply-ignored (not a reference flag) makes those five take effect as their
// help text describes: -r idx makes frame idx the cross-correlation reference (it
// is accumulated first, then the others in order); -k l:t and -s w:h crop
// every frame to that box before ingest (the box must lie inside the frame;
// any size the stack takes, 3 to 1024 per axis); --no-calcsum leaves out the
// sum images; --no-specklemasking leaves out bispectrum.dat, the phase
// reconstruction and the images made from it.  -f (follow) is not parsed by
// the reference (getopt prints the usage) and is not here either.
//
// Input: the reference decodes video/GIF with OpenCV (videoio.h:38-98); here
// <source> is an animated GIF (decoded by gif_decode.hpp into BGR frames, the
// order OpenCV delivers), a SER or uncompressed AVI recording (video_decode.hpp:
// 8 or 16-bit mono, or colour in BGR order), or a NumPy .npy frame stack,
// uint8/uint16/float32/float64, shape [frames][rows][cols] or
// [frames][rows][cols][channels].  For a
// multi-channel stack -c picks channel clamp(round(log2(c)), 0, channels-1)
// with r=1, g=2, b=4, i=7 (videoio.h:78-79), as Mat2Array does (so on BGR
// frames "r" reads the first channel, as the reference's does).
#include <getopt.h>

#include "gif_decode.hpp"
#include "video_decode.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "smip/gpu.hpp"

namespace {

int g_level = 1; // 0 notice, 1 info, 2 debug (the reference starts at info)

std::ostream& info()
{
    static std::ostream null(nullptr);
    return g_level >= 1 ? (std::cerr << "[info] ") : null;
}
std::ostream& notice() { return std::cerr << "[notice] "; }

void usage(const char* progname)
{
    std::cout << "   Usage :  " << progname << " [nrpbcvh?] <source root>\n"
              << "    available options:\n"
              << "     -n   --nrframes    <pics>    :   process at most number of <pics> frames\n"
              << "                                      default : all frames\n"
              << "     -r   --refframe    <index>   :   index of reference frame (default : first found)\n"
              << "     -p   --recoradius  <pixels>  :   radius of phase reconstruction (default : 2 * bispectrum extent)\n"
              << "     -b   --bdepth       <pixels>  :   bispectrum extent (3rd and 4th dimension) (default : 20)\n"
              << "     -c   --channel     <r|g|b|i> :   color channel (default: i)\n"
              << "          --calcsum               :   calculate picture sum and shifted sum (default)\n"
              << "          --no-calcsum            :   do not calculate picture sum and shifted sum\n"
              << "          --specklemasking        :   perform speckle masking (default)\n"
              << "          --no-specklemasking     :   do not perform speckle masking\n"
              << "     -k   --croppos <l:t>         :   fixed crop box position (default: 0:0)\n"
              << "     -s   --cropsize <w:h>        :   crop box size (default: total image)\n"
              << "     -v   --verbose               :   increase verbosity level\n"
              << "          --rings                 :   ring-parallel phase recovery (faster; not the reference's\n"
              << "                                      estimator: each spiral turn from earlier turns only)\n"
              << "          --apply-ignored         :   make -r, -k, -s, --no-calcsum and --no-specklemasking\n"
              << "                                      take effect (the reference parses and ignores them)\n"
              << "          --version               :   display version and exit\n"
              << "     -h -?  --help                :   help (this screen)\n"
              << "   <source root>: animated GIF, or NumPy .npy frame stack [frames][rows][cols](+[channels]),\n"
              << "                  uint8, uint16, float32 or float64\n\n";
}

// ------------------------------------------------------------ .npy reader
struct Npy {
    FILE* f = nullptr;
    char kind = 0; // 'u' or 'f'
    int esize = 0;
    std::vector<std::size_t> shape;
    long data_off = 0;
    std::vector<std::uint8_t> mem; // decoded frames (a GIF), used instead of the file when set
    std::shared_ptr<smipcli::VideoSource> video; // SER / AVI frames, read one at a time when set
    ~Npy()
    {
        if (f)
            std::fclose(f);
    }
};

void open_npy(Npy& n, const std::string& path)
{
    n.f = std::fopen(path.c_str(), "rb");
    if (!n.f)
        throw std::runtime_error("file open error: " + path);
    unsigned char magic[8];
    if (std::fread(magic, 1, 8, n.f) != 8 || std::memcmp(magic, "\x93NUMPY", 6) != 0)
        throw std::runtime_error(path + ": not a .npy file");
    std::size_t hlen = 0;
    if (magic[6] == 1) {
        unsigned char b[2];
        if (std::fread(b, 1, 2, n.f) != 2)
            throw std::runtime_error(path + ": truncated header");
        hlen = b[0] | (b[1] << 8);
    } else {
        unsigned char b[4];
        if (std::fread(b, 1, 4, n.f) != 4)
            throw std::runtime_error(path + ": truncated header");
        hlen = b[0] | (b[1] << 8) | (b[2] << 16) | ((std::size_t)b[3] << 24);
    }
    std::string h(hlen, '\0');
    if (std::fread(&h[0], 1, hlen, n.f) != hlen)
        throw std::runtime_error(path + ": truncated header");
    n.data_off = std::ftell(n.f);
    const auto descr = h.find("'descr'");
    const auto q = h.find('\'', h.find(':', descr) + 1);
    const std::string d = h.substr(q + 1, h.find('\'', q + 1) - q - 1); // e.g. "<u2", "|u1"
    if (d.size() < 3 || (d[0] != '<' && d[0] != '|' && d[0] != '='))
        throw std::runtime_error(path + ": unsupported dtype " + d + " (little-endian u1, u2, f4, f8 only)");
    n.kind = d[1];
    n.esize = std::atoi(d.c_str() + 2);
    const bool ok = (n.kind == 'u' && (n.esize == 1 || n.esize == 2)) || (n.kind == 'f' && (n.esize == 4 || n.esize == 8));
    if (!ok)
        throw std::runtime_error(path + ": unsupported dtype " + d + " (u1, u2, f4, f8)");
    if (h.find("'fortran_order': True") != std::string::npos)
        throw std::runtime_error(path + ": Fortran-ordered arrays are not supported");
    const auto s0 = h.find('(', h.find("'shape'"));
    const auto s1 = h.find(')', s0);
    std::stringstream ss(h.substr(s0 + 1, s1 - s0 - 1));
    std::string tok;
    while (std::getline(ss, tok, ','))
        if (tok.find_first_not_of(" ") != std::string::npos)
            n.shape.push_back(std::stoull(tok));
    if (n.shape.size() != 3 && n.shape.size() != 4)
        throw std::runtime_error(path + ": expected [frames][rows][cols] or [frames][rows][cols][channels]");
}

// ------------------------------------------------------------- PNG writer
// 16-bit gray or RGB, zlib stream of stored (uncompressed) deflate blocks.
uint32_t crc32(const unsigned char* p, std::size_t n, uint32_t c = 0xffffffffu)
{
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k)
                v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            table[i] = v;
        }
        init = true;
    }
    for (std::size_t i = 0; i < n; ++i)
        c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c;
}

void put32(std::vector<unsigned char>& v, uint32_t x)
{
    v.push_back(x >> 24);
    v.push_back(x >> 16);
    v.push_back(x >> 8);
    v.push_back(x);
}

void write_chunk(FILE* f, const char* type, const std::vector<unsigned char>& data)
{
    std::vector<unsigned char> c;
    put32(c, (uint32_t)data.size());
    c.insert(c.end(), type, type + 4);
    c.insert(c.end(), data.begin(), data.end());
    const uint32_t crc = crc32(c.data() + 4, c.size() - 4) ^ 0xffffffffu;
    put32(c, crc);
    std::fwrite(c.data(), 1, c.size(), f);
}

void write_png16(const std::string& path, std::size_t w, std::size_t h, int channels, const std::vector<uint16_t>& px)
{
    std::vector<unsigned char> raw;
    raw.reserve(h * (1 + w * channels * 2));
    for (std::size_t y = 0; y < h; ++y) {
        raw.push_back(0); // filter: none
        for (std::size_t x = 0; x < w * channels; ++x) {
            const uint16_t v = px[y * w * channels + x];
            raw.push_back(v >> 8);
            raw.push_back(v & 0xff);
        }
    }
    std::vector<unsigned char> z { 0x78, 0x01 };
    uint32_t a = 1, b = 0;
    for (unsigned char c : raw) {
        a = (a + c) % 65521;
        b = (b + a) % 65521;
    }
    for (std::size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const std::size_t len = std::min<std::size_t>(65535, raw.size() - off);
        z.push_back(off + len >= raw.size() ? 1 : 0);
        z.push_back(len & 0xff);
        z.push_back(len >> 8);
        z.push_back(~len & 0xff);
        z.push_back((~len >> 8) & 0xff);
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        if (raw.empty())
            break;
    }
    put32(z, (b << 16) | a);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f)
        throw std::runtime_error("unable to open " + path + " for writing");
    static const unsigned char sig[8] = { 0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n' };
    std::fwrite(sig, 1, 8, f);
    std::vector<unsigned char> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.push_back(16);                       // bit depth
    ihdr.push_back(channels == 3 ? 2 : 0);    // colour type: RGB or gray
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    write_chunk(f, "IHDR", ihdr);
    write_chunk(f, "IDAT", z);
    write_chunk(f, "IEND", {});
    std::fclose(f);
}

// Array2Mat (videoio.h:100-156): pixel (x, y) shows element (x + min_x, y +
// min_y) of the signed index range when signed_symmetry (an fftshift), scaled
// by 65535 (gray) or through mapToColor (videoio.h:178-206, false colour).
// The reference's static_cast of values outside [0, 1] to uint16 is undefined;
// they are clamped here.
template <class F>
void save_image(const std::string& path, std::size_t w, std::size_t h, F value, bool signed_symmetry, bool colour)
{
    std::vector<uint16_t> px(w * h * (colour ? 3 : 1));
    const long hx = (long)(w >> 1), hy = (long)(h >> 1);
    for (std::size_t y = 0; y < h; ++y)
        for (std::size_t x = 0; x < w; ++x) {
            std::size_t sx = x, sy = y;
            if (signed_symmetry) {
                sx = (std::size_t)(((long)x - hx + (long)w) % (long)w);
                sy = (std::size_t)(((long)y - hy + (long)h) % (long)h);
            }
            const double v = value(sx, sy);
            if (!colour) {
                const double s = v * 65535.0;
                px[y * w + x] = (uint16_t)(s >= 65535.0 ? 65535.0 : (s > 0.0 ? s : 0.0));
            } else {
                const double c = std::clamp(std::isnan(v) ? 0.0 : v, 0., 1.);
                const double M = 65535.0;
                double r, g, b;
                if (c < 0.25) {
                    r = 0; g = 0; b = M * (4 * c);
                } else if (c < 0.5) {
                    r = 0; g = M * (4 * c - 1); b = M * (2 - 4 * c);
                } else if (c < 0.75) {
                    r = M * (4 * c - 2); g = M * (3 - 4 * c); b = 0;
                } else {
                    r = M; g = 0; b = M * (4 * c - 3);
                }
                px[3 * (y * w + x)] = (uint16_t)r;
                px[3 * (y * w + x) + 1] = (uint16_t)g;
                px[3 * (y * w + x) + 2] = (uint16_t)b;
            }
        }
    write_png16(path, w, h, colour ? 3 : 1, px);
}

// Crop box of the frames handed to the stack: columns [l, l + w), rows [t, t + h).
struct Crop {
    std::size_t l = 0, t = 0, w = 0, h = 0;
};

// Pushes frames order[first, first + count) of the source, channel `channel`,
// cut to the crop box.
template <class T>
void push_chunk(smip::gpu::Stack& st, Npy& n, const std::vector<std::size_t>& order, std::size_t first,
                std::size_t count, std::size_t channel, const Crop& cr)
{
    const std::size_t rows = n.shape[1], cols = n.shape[2];
    const std::size_t ch = n.shape.size() == 4 ? n.shape[3] : 1;
    const std::size_t fe = rows * cols * ch;
    std::vector<T> in(fe);
    std::vector<T> out(cr.w * cr.h * count);
    for (std::size_t k = 0; k < count; ++k) {
        const std::size_t idx = order[first + k];
        if (n.video) {
            n.video->read_frame(idx, in.data());
        } else if (!n.mem.empty()) {
            std::memcpy(in.data(), n.mem.data() + idx * fe * sizeof(T), fe * sizeof(T));
        } else {
            std::fseek(n.f, n.data_off + (long)(idx * fe * sizeof(T)), SEEK_SET);
            if (std::fread(in.data(), sizeof(T), fe, n.f) != fe)
                throw std::runtime_error("error reading frames");
        }
        T* o = out.data() + k * cr.w * cr.h;
        for (std::size_t y = 0; y < cr.h; ++y)
            for (std::size_t x = 0; x < cr.w; ++x)
                o[y * cr.w + x] = in[((cr.t + y) * cols + cr.l + x) * ch + channel];
    }
    st.push_frames(out.data(), count);
}

} // namespace

int main(int argc, char* argv[])
{
    const char* progname = argv[0];
    std::size_t max_frames { 10'000 };
    std::size_t bispectrum_depth { 20 };
    std::size_t reco_radius = bispectrum_depth * 2;
    int color_channel = 7; // white
    int swSpeckleMasking { 1 };
    int swCalcSum { 1 };
    int swShowVersion { 0 };
    int swApplyIgnored { 0 };
    int swRings { 0 };
    std::size_t ref_frame { 0 };
    long crop_l = -1, crop_t = -1, crop_w = -1, crop_h = -1;
    std::size_t verbose { 0 };
    try {
        for (int ch = 0; ch != -1;) {
            static struct option long_options[] = {
                { "verbose", no_argument, 0, 'v' },
                { "bdepth", required_argument, 0, 'b' },
                { "recoradius", required_argument, 0, 'p' },
                { "refframe", required_argument, 0, 'r' },
                { "nrframes", required_argument, 0, 'n' },
                { "channel", required_argument, 0, 'c' },
                { "croppos", required_argument, 0, 'k' },
                { "cropsize", required_argument, 0, 's' },
                { "help", no_argument, 0, 'h' },
                { "version", no_argument, &swShowVersion, 1 },
                { "no-calcsum", no_argument, &swCalcSum, 0 },
                { "calcsum", no_argument, &swCalcSum, 1 },
                { "no-specklemasking", no_argument, &swSpeckleMasking, 0 },
                { "specklemasking", no_argument, &swSpeckleMasking, 1 },
                { "apply-ignored", no_argument, &swApplyIgnored, 1 },
                { "rings", no_argument, &swRings, 1 },
                { 0, 0, 0, 0 }
            };
            int option_index { 0 };
            ch = getopt_long(argc, argv, "vn:r:p:b:c:h?k:s:", long_options, &option_index);
            std::istringstream istr;
            switch (ch) {
            case 'v': verbose++; break;
            case 'n': max_frames = std::strtoul(optarg, nullptr, 10); break;
            case 'r': ref_frame = std::strtoul(optarg, nullptr, 10); break; // unused by the reference (main.cpp:132-134)
            case 'p': reco_radius = std::strtoul(optarg, nullptr, 10); break;
            case 'b': bispectrum_depth = std::strtoul(optarg, nullptr, 10); break;
            case 'k': {
                istr.str(std::string(optarg));
                int a = -1, b = -1;
                char c;
                istr >> a >> c >> b;
                if (a < 0 || b < 0)
                    throw std::range_error("invalid crop box pos arguments");
                crop_l = a;
                crop_t = b;
                break; // unused by the reference (main.cpp:146-156)
            }
            case 's': {
                istr.str(std::string(optarg));
                int a = -1, b = -1;
                char c;
                istr >> a >> c >> b;
                if (a <= 0 || b <= 0)
                    throw std::range_error("invalid crop box size arguments");
                crop_w = a;
                crop_h = b;
                break; // unused by the reference (main.cpp:157-167)
            }
            case 'c': {
                const std::string s(optarg);
                for (char c : s) {
                    if (c == 'r') color_channel = 1;
                    else if (c == 'g') color_channel = 2;
                    else if (c == 'b') color_channel = 4;
                    else if (c == 'i') color_channel = 7;
                }
                break;
            }
            case 'h':
            case '?': usage(progname); return 0;
            default: break;
            }
        }
        if (swShowVersion) {
            int a = 0, b = 0, c = 0;
            smip_version(&a, &b, &c);
            std::cout << "Speckle Masking Image Processing v" << a << "." << b << "." << c << " (GB300)" << std::endl;
            return 0;
        }
        g_level = verbose >= 2 ? 2 : 1;
        argc -= optind;
        argv += optind;
        if (argc != 1) {
            usage(progname);
            return 0;
        }
        if (!swApplyIgnored) { // the reference's behaviour: these flags change nothing
            ref_frame = 0;
            crop_l = crop_t = crop_w = crop_h = -1;
            swCalcSum = swSpeckleMasking = 1;
        }
        const std::string filename(*argv);

        Npy npy;
        if (smipcli::is_gif(filename)) {
            // animated GIF: frames in BGR, as OpenCV's VideoCapture delivers them
            smipcli::GifFrames gf = smipcli::read_gif(filename, max_frames);
            npy.kind = 'u';
            npy.esize = 1;
            npy.shape = { gf.count, gf.height, gf.width, 3 };
            npy.mem = std::move(gf.bgr);
        } else if (smipcli::VideoSource::is_ser(filename) || smipcli::VideoSource::is_avi(filename)) {
            // SER / uncompressed AVI: one channel, or three in B, G, R order; 8 or 16-bit samples
            auto v = std::make_shared<smipcli::VideoSource>(smipcli::VideoSource::is_ser(filename)
                                                                ? smipcli::VideoSource::open_ser(filename)
                                                                : smipcli::VideoSource::open_avi(filename));
            npy.kind = 'u';
            npy.esize = v->esize;
            npy.shape = { v->count, v->height, v->width };
            if (v->channels > 1)
                npy.shape.push_back(v->channels);
            npy.video = v;
        } else {
            open_npy(npy, filename);
        }
        info() << "opened frame stack " << filename << ": " << npy.shape[0] << " frames\n";
        const std::size_t nframes = std::min<std::size_t>(npy.shape[0], max_frames);
        notice() << "using " << nframes << "/" << npy.shape[0] << " frames\n";
        if (nframes == 0)
            throw std::runtime_error("no frames");
        const std::size_t src_rows = npy.shape[1], src_cols = npy.shape[2];
        const std::size_t nch = npy.shape.size() == 4 ? npy.shape[3] : 1;
        const long chan = std::clamp<long>(std::lround(std::log2((double)color_channel)), 0L, (long)nch - 1);
        Crop cr { 0, 0, src_cols, src_rows };
        if (crop_l >= 0) {
            cr.l = (std::size_t)crop_l;
            cr.t = (std::size_t)crop_t;
        }
        if (crop_w > 0) {
            cr.w = (std::size_t)crop_w;
            cr.h = (std::size_t)crop_h;
        } else {
            cr.w = src_cols > cr.l ? src_cols - cr.l : 0;
            cr.h = src_rows > cr.t ? src_rows - cr.t : 0;
        }
        if (cr.w == 0 || cr.h == 0 || cr.l + cr.w > src_cols || cr.t + cr.h > src_rows)
            throw std::range_error("crop box outside the frame");
        if (ref_frame >= nframes)
            throw std::range_error("reference frame index out of range");
        // accumulation order: the reference frame first, then the others in order
        std::vector<std::size_t> order;
        order.reserve(nframes);
        order.push_back(ref_frame);
        for (std::size_t i = 0; i < nframes; ++i)
            if (i != ref_frame)
                order.push_back(i);
        const std::size_t rows = cr.h, cols = cr.w;

        info() << "creating bispectrum with size [" << cols << " " << rows << " " << bispectrum_depth << " "
               << bispectrum_depth << "]\n";
        smip::gpu::Stack st(cols, rows, bispectrum_depth);
        info() << "accumulating sum, power spectrum and bispectrum of all frames\n";
        const std::size_t chunk = 256;
        for (std::size_t f0 = 0; f0 < nframes; f0 += chunk) {
            const std::size_t k = std::min(chunk, nframes - f0);
            const std::size_t c = (std::size_t)chan;
            if (npy.kind == 'u' && npy.esize == 1) push_chunk<std::uint8_t>(st, npy, order, f0, k, c, cr);
            else if (npy.kind == 'u') push_chunk<std::uint16_t>(st, npy, order, f0, k, c, cr);
            else if (npy.esize == 4) push_chunk<float>(st, npy, order, f0, k, c, cr);
            else push_chunk<double>(st, npy, order, f0, k, c, cr);
        }
        if (g_level >= 2) {
            const auto sh = st.shifts();
            for (std::size_t i = 0; i < sh.size(); ++i)
                std::cerr << "[debug] frame " << order[i] << " relative shift wrt ref frame: [x,y] = [" << sh[i][0]
                          << "," << sh[i][1] << "]\n";
        }
        smip::gpu::Image<double> sum = st.sum();
        smip::gpu::Image<double> power = st.power();
        // main.cpp:359-376: power / (max / 1000); sum / 255
        double pmax = 0.0;
        for (double v : power)
            pmax = std::max(pmax, std::abs(v));
        const double normfact = pmax / 1000.;
        for (double& v : power)
            v /= normfact;
        for (double& v : sum)
            v /= 255.;
        if (swCalcSum) {
            save_image("sum_image_falsecolor.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::fabs(sum(x, y)); }, false, true);
            save_image("sum_image.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::fabs(sum(x, y)); }, false, false);
        }
        if (swSpeckleMasking) {
            notice() << "writing bispectrum to file 'bispectrum.dat'\n";
            st.write_to_file("bispectrum.dat");

            info() << "reconstructing fourier phases from bispectrum\n";
            if (swRings)
                st.set_reco_mode(SMIP_RECO_RINGS);
            const auto res = st.finish((double)reco_radius);
            // main.cpp:329-331: phases windowed by Hann of aperture 2R for the outputs
            const auto win = smip::gpu::Hann<double>(cols, rows, (double)reco_radius * 2);
            smip::gpu::Image<std::complex<double>> phases = res.phases;
            for (std::size_t i = 0; i < phases.size(); ++i)
                phases.data()[i] *= win.data()[i];
            auto phase01 = [](std::complex<double> z) { return (std::arg(z) + M_PI) / (2 * M_PI); };
            save_image("phases_falsecolor.png", cols, rows, [&](std::size_t x, std::size_t y) { return phase01(phases(x, y)); }, true, true);
            save_image("phases.png", cols, rows, [&](std::size_t x, std::size_t y) { return phase01(phases(x, y)); }, true, false);
            save_image("phasecons.png", cols, rows, [&](std::size_t x, std::size_t y) { return res.pm.consistency(x, y); }, true, true);
            save_image("powerspec_falsecolor.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::fabs(power(x, y)); }, true, true);
            save_image("powerspec.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::fabs(power(x, y)); }, true, false);
            save_image("reco_image_falsecolor.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::abs(res.image(x, y)); }, true, true);
            save_image("reco_image.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::abs(res.image(x, y)); }, true, false);
        } else {
            save_image("powerspec_falsecolor.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::fabs(power(x, y)); }, true, true);
            save_image("powerspec.png", cols, rows, [&](std::size_t x, std::size_t y) { return std::fabs(power(x, y)); }, true, false);
        }
        info() << "done\n";
    } catch (const std::exception& e) {
        std::cerr << "[critical] " << e.what() << "\n";
        return 1;
    }
    return 0;
}
