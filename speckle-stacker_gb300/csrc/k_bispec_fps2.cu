// k_bispec_fps2.cu -- the bispectrum kernel with two frames per ring stage
// (k_bispec.cuh), a variant the autotuner may choose per shape.  Its own
// translation unit keeps the library's build parallel.
#include "k_bispec.cuh"

namespace smip_gpu {

cudaError_t launch_bispec_accumulate_fps2(const BispecLaunch& L, const Geometry& g, cudaStream_t st)
{
    return launch_variant<2>(L, g, st);
}

} // namespace smip_gpu
