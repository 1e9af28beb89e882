// k_finish.cu -- final reconstruction in FP64.
//
// Replaces smip-cli/main.cpp:328-376: Hann window on the phases
// (window_function.h:70-85 with alpha 0.5, aperture 2*reco_radius),
// sqrt(power spectrum) x phases, FFTW backward transform (unnormalised) and
// division of the image by its largest modulus.  Operation order follows the
// reference's complex arithmetic so only rounding differs.
#include "smip_dev.cuh"

namespace smip_gpu {

// FFT-order index x -> the signed index of Array2's range [-(n/2), n - n/2 - 1]
// (include/array2.h:310-339); for odd n the upper half is one longer.
__device__ __forceinline__ int signed_idx(int x, int n) { return x < n - n / 2 ? x : x - n; }

// power at FFT-order (x, y) from the u_x <= 0 half plane P[a][c]
__device__ __forceinline__ double power_at(const double* Ph, int sx, int sy, int H)
{
    int a, c;
    if (sx <= 0) {
        a = -sx;
        c = sy + H / 2;
    } else { // P(x, y) = P(-x, -y)
        a = sx;
        c = H / 2 - sy; // y = -sy, wrapped into [-(H/2), H - 1 - H/2]
        if (c >= H)
            c -= H;
    }
    return Ph[(long long)a * H + c];
}

__global__ void finish_build_kernel(const double* __restrict__ Ph, double pnorm, const double2* __restrict__ phases,
                                    double trigarg, int W, int H, double2* __restrict__ Z, double* __restrict__ pfull)
{
    const int n = W * H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int sx = signed_idx(p % W, W), sy = signed_idx(p / W, H);
        const double pn = power_at(Ph, sx, sy, H) / pnorm;
        if (pfull)
            pfull[p] = pn;
        if (Z) {
            const double w = (0.5 + 0.5 * cos(trigarg * (double)sx)) * (0.5 + 0.5 * cos(trigarg * (double)sy));
            const double2 ph = phases[p];
            const double wr = ph.x * w - ph.y * 0.0, wi = ph.x * 0.0 + ph.y * w;
            const double s = sqrt(pn);
            Z[p] = make_double2(s * wr - 0.0 * wi, s * wi + 0.0 * wr);
        }
    }
}

__global__ void hann_kernel(double* __restrict__ out, int W, int H, double trigarg)
{
    const int n = W * H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int sx = signed_idx(p % W, W), sy = signed_idx(p / W, H);
        out[p] = (0.5 + 0.5 * cos(trigarg * (double)sx)) * (0.5 + 0.5 * cos(trigarg * (double)sy));
    }
}

// Batched in-place FFT of lines of length 2^logn (element stride es, line
// stride ls), double precision, 4 lines per CTA.
__global__ void __launch_bounds__(256) fft_lines_d_kernel(double2* __restrict__ data, int logn, int nlines, long long ls,
                                                           long long es, int sign, const double2* __restrict__ tw_g)
{
    extern __shared__ double2 smd[];
    double2* tw = smd;
    double2* L = smd + (1 << (kTwLog - 1));
    const int n = 1 << logn;
    const int l0 = blockIdx.x * 4;
    const int nl = min(4, nlines - l0);
    load_twiddles(tw, tw_g, kTwLog);
    for (int idx = threadIdx.x; idx < nl * n; idx += blockDim.x) {
        const int l = idx >> logn, k = idx & (n - 1);
        L[l * n + bitrev(k, logn)] = data[(l0 + l) * ls + k * es];
    }
    __syncthreads();
    fft_stages(L, logn, nl, n, tw, kTwLog, sign);
    for (int idx = threadIdx.x; idx < nl * n; idx += blockDim.x) {
        const int l = idx >> logn, k = idx & (n - 1);
        data[(l0 + l) * ls + k * es] = L[l * n + k];
    }
}

// max |Z| over the grid: per-block maxima combined with an integer atomicMax
// on the bit patterns (non-negative doubles order like their bits), so the
// result does not depend on block order; *out must be zero beforehand.
__global__ void max_abs_kernel(const double2* __restrict__ Z, int n, double* out)
{
    __shared__ double red[32];
    double m = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const double2 z = Z[p];
        m = fmax(m, hypot(z.x, z.y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i)
            r = fmax(r, red[i]);
        atomicMax(reinterpret_cast<unsigned long long*>(out), (unsigned long long)__double_as_longlong(r));
    }
}

__global__ void scale_kernel(double2* __restrict__ Z, int n, const double* __restrict__ m)
{
    const double d = *m;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const double2 z = Z[p];
        Z[p] = make_double2(z.x / d, z.y / d);
    }
}

static int grid_n(int n) { return (n + 255) / 256 < 2048 ? (n + 255) / 256 : 2048; }

cudaError_t launch_finish(const double* Phalf, double pnorm, const double2* phases, double aperture, const Geometry& g,
                          double2* Z, double* power_full, double* maxbuf, const double2* tw64, cudaStream_t st,
                          const double2* twW64, const double2* twH64)
{
    const int n = g.W * g.H;
    const double trigarg = 6.283185307179586476925286766559 / aperture;
    finish_build_kernel<<<grid_n(n), 256, 0, st>>>(Phalf, pnorm, phases, trigarg, g.W, g.H, Z, power_full); note_launches(1);
    cudaError_t e = cudaSuccess;
    if (g.generic) { // FFTW_BACKWARD over rows (x) then columns (y), mixed radix
        if ((e = launch_gen_lines_d(Z, g.pW, g.H, g.W, 1, +1, twW64, st)) != cudaSuccess
            || (e = launch_gen_lines_d(Z, g.pH, g.W, 1, g.W, +1, twH64, st)) != cudaSuccess)
            return e;
    } else {
        const size_t smem = sizeof(double2) * ((1 << (kTwLog - 1)) + 4 * (size_t)(g.W > g.H ? g.W : g.H));
        // the limit is the largest frame's, so that concurrent launches of other shapes never lower it
        const size_t smem_max = sizeof(double2) * ((1 << (kTwLog - 1)) + 4 * (size_t)(1 << kMaxLog));
        e = cudaFuncSetAttribute(fft_lines_d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        if (e != cudaSuccess)
            return e;
        // FFTW_BACKWARD over rows (x) then columns (y)
        fft_lines_d_kernel<<<(g.H + 3) / 4, 256, smem, st>>>(Z, g.logW, g.H, g.W, 1, +1, tw64); note_launches(1);
        fft_lines_d_kernel<<<(g.W + 3) / 4, 256, smem, st>>>(Z, g.logH, g.W, 1, g.W, +1, tw64); note_launches(1);
    }
    if ((e = cudaMemsetAsync(maxbuf, 0, sizeof(double), st)) != cudaSuccess)
        return e;
    max_abs_kernel<<<(n + 255) / 256 < 256 ? (n + 255) / 256 : 256, 256, 0, st>>>(Z, n, maxbuf); note_launches(1);
    scale_kernel<<<grid_n(n), 256, 0, st>>>(Z, n, maxbuf); note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_power_full(const double* Phalf, double pnorm, const Geometry& g, double* power_full,
                              cudaStream_t st)
{
    const int n = g.W * g.H;
    finish_build_kernel<<<grid_n(n), 256, 0, st>>>(Phalf, pnorm, nullptr, 0.0, g.W, g.H, nullptr, power_full); note_launches(1);
    return cudaGetLastError();
}

// Array2<double>::shifted(distance) (array2.h:603-622): element (x, y) of the
// result is in(x - dx, y - dy), zero where that lies outside.  For |dx| < W and
// |dy| < H this is exactly the reference's clamped copy range.
__global__ void shifted_kernel(const double* __restrict__ in, double* __restrict__ out, int W, int H, int dx, int dy)
{
    const int n = W * H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int x = i % W, y = i / W;
        const int sx = x - dx, sy = y - dy;
        out[i] = (sx >= 0 && sx < W && sy >= 0 && sy < H) ? in[sx + sy * W] : 0.0;
    }
}

cudaError_t launch_shifted(const double* in, double* out, int W, int H, int dx, int dy, cudaStream_t st)
{
    const int n = W * H;
    shifted_kernel<<<grid_n(n), 256, 0, st>>>(in, out, W, H, dx, dy); note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_hann(double* out, int W, int H, double aperture, cudaStream_t st)
{
    const int n = W * H;
    hann_kernel<<<grid_n(n), 256, 0, st>>>(out, W, H, 6.283185307179586476925286766559 / aperture); note_launches(1);
    return cudaGetLastError();
}

} // namespace smip_gpu
