// Decodes a GIF with smip-cli's decoder and writes the frames as raw BGR
// bytes; prints "count height width".  Used by tests/test_gif.py.
#include "gif_decode.hpp"

#include <cstdio>

int main(int argc, char** argv)
{
    if (argc != 3)
        return 2;
    try {
        const smipcli::GifFrames g = smipcli::read_gif(argv[1]);
        std::printf("%zu %zu %zu\n", g.count, g.height, g.width);
        FILE* f = std::fopen(argv[2], "wb");
        if (!f || std::fwrite(g.bgr.data(), 1, g.bgr.size(), f) != g.bgr.size())
            return 3;
        std::fclose(f);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
