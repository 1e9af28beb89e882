// Reads a SER or AVI file with smip-cli's decoder and writes every frame as
// raw bytes (host byte order); prints "count height width channels esize".
// Used by tests/test_video.py.
#include "video_decode.hpp"

#include <cstdio>
#include <vector>

int main(int argc, char** argv)
{
    if (argc != 3)
        return 2;
    try {
        const std::string path = argv[1];
        const smipcli::VideoSource v = smipcli::VideoSource::is_ser(path) ? smipcli::VideoSource::open_ser(path)
                                                                           : smipcli::VideoSource::open_avi(path);
        std::printf("%zu %zu %zu %zu %d\n", v.count, v.height, v.width, v.channels, v.esize);
        std::vector<unsigned char> buf(v.height * v.width * v.channels * v.esize);
        FILE* f = std::fopen(argv[2], "wb");
        if (!f)
            return 3;
        for (std::size_t k = 0; k < v.count; ++k) {
            v.read_frame(k, buf.data());
            if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size())
                return 3;
        }
        std::fclose(f);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
