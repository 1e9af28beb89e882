// k_bispec.cu -- bispectrum accumulation launches (the kernel is in
// k_bispec.cuh), the Kahan normalise / merge kernels and the bounded-wait
// diagnostic.
#include "k_bispec.cuh"

namespace smip_gpu {

bool bispec_depth_supported(int De) { return De >= 2 && De <= 64 && De % 2 == 0; }

// partial sums of one split-tile part: (8 j x 4 l + 1 edge) float2 per thread, 512 threads
size_t bispec_scratch_bytes(int num_sms) { return (size_t)num_sms * kCtasPerSm * 33 * (512 / kCtasPerSm) * sizeof(float2); }
size_t bispec_tile_counters(int num_sms) { return (size_t)num_sms * kCtasPerSm; }

// The staging variant the stack's tuning chose: four frames per ring stage
// (here), or two (k_bispec_fps2.cu).
cudaError_t launch_bispec_accumulate(const BispecLaunch& L, const Geometry& g, cudaStream_t st)
{
    if (L.nframes <= 0)
        return cudaSuccess;
    if (L.variant == 1)
        return launch_bispec_accumulate_fps2(L, g, st);
    return launch_variant<4>(L, g, st);
}

// ------------------------------------------------ bounded-wait diagnostic
// The failure path every kernel takes when a wait expires, run on purpose:
// block 0 waits (bounded, as the bispectrum kernel's ring does) on an mbarrier
// that nothing arrives on; block 1 polls (bounded, as the phase walk does) a
// global flag that nothing sets.  Both record SMIP_DEV_ERR_TIMEOUT and return;
// no copy is in flight and nothing else waits on them.
__global__ void bounded_wait_probe_kernel(int* err, unsigned long long timeout_ns, const int* never)
{
    __shared__ __align__(8) uint64_t bar;
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) {
            mbar_init(&bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        const bool got = mbar_wait_bounded(&bar, 0, timeout_ns);
        if (!__all_sync(0xffffffffu, got) && threadIdx.x == 0)
            record_error(err, SMIP_DEV_ERR_TIMEOUT);
    } else {
        const unsigned long long t0 = globaltimer_ns();
        bool got = false;
        while (!(got = *reinterpret_cast<const volatile int*>(never) != 0) && globaltimer_ns() - t0 <= timeout_ns) {
        }
        if (!got && threadIdx.x == 0)
            record_error(err, SMIP_DEV_ERR_TIMEOUT);
    }
}

cudaError_t launch_bounded_wait_probe(int* err, const int* never, double timeout_s, cudaStream_t st)
{
    bounded_wait_probe_kernel<<<2, 32, 0, st>>>(err, (unsigned long long)(timeout_s * 1e9), never);
    note_launches(1);
    return cudaGetLastError();
}

// ------------------------------------------------------- normalise, merge
// (B - C) / n: the difference is exact in FP64; a multiply by 1/n instead of
// a divide keeps the FP64 pipe's share small (GB300's FP64 rate is low).
__global__ void bispec_normalize_kernel(const float2* __restrict__ B, const float2* __restrict__ C, double inv_n,
                                        long long count, float2* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const float2 b = B[i], c = C[i];
        out[i] = make_float2((float)(((double)b.x - (double)c.x) * inv_n), (float)(((double)b.y - (double)c.y) * inv_n));
    }
}

// dst += src, both Kahan pairs: the src sum (b - c) is added with compensation.
__global__ void bispec_merge_kernel(float2* __restrict__ Bd, float2* __restrict__ Cd, const float2* __restrict__ Bs,
                                    const float2* __restrict__ Cs, long long count)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        float2 b = Bd[i], c = Cd[i];
        const float2 sb = Bs[i], sc = Cs[i];
        const float vx = sb.x - sc.x, vy = sb.y - sc.y;
        const float yx = vx - c.x, yy = vy - c.y;
        const float tx = b.x + yx, ty = b.y + yy;
        c.x = (tx - b.x) - yx;
        c.y = (ty - b.y) - yy;
        Bd[i] = make_float2(tx, ty);
        Cd[i] = c;
    }
}

cudaError_t launch_bispec_normalize(const float2* B, const float2* C, double nframes, long long n, float2* out,
                                    cudaStream_t st)
{
    bispec_normalize_kernel<<<2048, 256, 0, st>>>(B, C, 1.0 / nframes, n, out); note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_bispec_merge(float2* Bd, float2* Cd, const float2* Bs, const float2* Cs, long long n,
                                cudaStream_t st)
{
    bispec_merge_kernel<<<2048, 256, 0, st>>>(Bd, Cd, Bs, Cs, n); note_launches(1);
    return cudaGetLastError();
}

} // namespace smip_gpu
