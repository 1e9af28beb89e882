// k_xcorr.cu -- integer shift of each frame against frame 0, and the
// shift-and-add sum.
//
// Replaces CrossCorrelation::calculate_displacement (include/crosscorrel.h:
// 166-179: first maximum of the FP64 FFT correlation in row-major order,
// wrapped to a signed shift) and the sumarray update of smip-cli/main.cpp:
// 289-294 with Array2::shifted (include/array2.h:603-622).
//
// The correlation arrives in FP32 (k_fft.cu).  Every position within an
// error bound of the FP32 peak is re-scored exactly -- integer arithmetic for
// u8/u16 frames, FP64 for float frames -- and the best exact value wins, ties
// to the lowest linear index (std::max_element's first maximum).  The bound
// is 8 * 2^-24 * log2(W*H) * ||ref||_2 * ||frame||_2 * W*H, a few times the
// worst-case error of an FP32 radix-2 FFT convolution (for mixed-radix
// transforms the sum of the factors of W and H takes the place of log2(W*H)).
#include <cstdint>

#include "smip_dev.cuh"

namespace smip_gpu {

constexpr int kShiftThreads = 512;
constexpr int kMaxCand = 1024;

template <typename T> struct ExactAcc { using type = double; };
template <> struct ExactAcc<uint8_t> { using type = unsigned long long; };
template <> struct ExactAcc<uint16_t> { using type = unsigned long long; };

template <typename A>
__device__ A block_sum(A v, A* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        red[w] = v;
    __syncthreads();
    A s = 0;
    for (int i = 0; i < nw; ++i)
        s += red[i];
    return s;
}

template <typename A, typename T> __device__ __forceinline__ A mul_exact(T a, T b) { return (A)a * (A)b; }
template <> __device__ __forceinline__ unsigned long long mul_exact<unsigned long long, uint16_t>(uint16_t a, uint16_t b)
{
    return (unsigned long long)((unsigned)a * (unsigned)b); // < 2^32, exact
}
template <> __device__ __forceinline__ unsigned long long mul_exact<unsigned long long, uint8_t>(uint8_t a, uint8_t b)
{
    return (unsigned long long)((unsigned)a * (unsigned)b);
}

constexpr int kMulti = 8; // candidates scored per sweep over the frame

// Exact correlations sum_p ref(p) frame((p + s_c) mod (W, H)) of up to kMulti
// candidate shifts s_c = cand[c] (row-major index) in one sweep.  Frames whose
// width is a power of two (logW >= 0) take four consecutive pixels per thread
// step with shifts and masks instead of divisions; other widths (logW = -1)
// one pixel per step with wrapped indices.  Results land in out[c] for every
// thread.
template <typename T>
__device__ void exact_corr_multi(const T* __restrict__ ref, const T* __restrict__ fr, int W, int logW, int H,
                                 const int* cand, int k, typename ExactAcc<T>::type* out,
                                 typename ExactAcc<T>::type* red /* [kMulti][32] */)
{
    using A = typename ExactAcc<T>::type;
    const int n = W * H;
    A acc[kMulti];
#pragma unroll
    for (int c = 0; c < kMulti; ++c)
        acc[c] = 0;
    int sx[kMulti], sy[kMulti];
#pragma unroll
    for (int c = 0; c < kMulti; ++c) {
        const int q = c < k ? cand[c] : 0;
        sx[c] = q % W;
        sy[c] = q / W;
    }
    const bool vec = (reinterpret_cast<uintptr_t>(ref) & 15) == 0;
    if (logW < 0) {
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
            const int y = p / W, x = p - y * W;
            const T r = ref[p];
#pragma unroll
            for (int c = 0; c < kMulti; ++c) {
                if (c < k) {
                    int ys = y + sy[c], xs = x + sx[c];
                    ys -= ys >= H ? H : 0;
                    xs -= xs >= W ? W : 0;
                    acc[c] += mul_exact<A>(r, fr[ys * W + xs]);
                }
            }
        }
    }
    for (int p = threadIdx.x * 4; logW >= 0 && p < n; p += blockDim.x * 4) {
        const int x = p & (W - 1), y = p >> logW;
        T r4[4];
        if (vec && sizeof(T) == 1)
            *reinterpret_cast<uint32_t*>(r4) = *reinterpret_cast<const uint32_t*>(ref + p);
        else if (vec && sizeof(T) == 2)
            *reinterpret_cast<uint2*>(r4) = *reinterpret_cast<const uint2*>(ref + p);
        else if (vec && sizeof(T) == 4)
            *reinterpret_cast<uint4*>(r4) = *reinterpret_cast<const uint4*>(ref + p);
        else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                r4[e] = ref[p + e];
        }
#pragma unroll
        for (int c = 0; c < kMulti; ++c) {
            if (c < k) {
                const T* row = fr + (((y + sy[c]) & (H - 1)) << logW);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    acc[c] += mul_exact<A>(r4[e], row[(x + e + sx[c]) & (W - 1)]);
            }
        }
    }
    // block reduction of the k sums at once
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < kMulti; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    }
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < kMulti; ++c)
            red[c * 32 + w] = acc[c];
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kMulti; ++c) {
        A t = 0;
        for (int i = 0; i < nw; ++i)
            t += red[c * 32 + i];
        out[c] = t;
    }
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kShiftThreads) xcorr_shift_kernel(const float* __restrict__ corr,
                                                                     const float* __restrict__ rowmax,
                                                                     const T* __restrict__ frames, long long fstride,
                                                                     const T* __restrict__ ref, const double* ref_sq,
                                                                     int first_is_frame0, int W, int logW, int H,
                                                                     double err_stages, int* __restrict__ shifts)
{
    using A = typename ExactAcc<T>::type;
    __shared__ A redM[kMulti * 32];
    __shared__ A redA1[32];
    __shared__ float redF[32];
    __shared__ int cand[kMaxCand];
    __shared__ int ncand;
    const int f = blockIdx.x;
    if (first_is_frame0 && f == 0) {
        if (threadIdx.x == 0) {
            shifts[0] = 0;
            shifts[1] = 0;
        }
        return;
    }
    const int n = W * H;
    const float* c = corr + (long long)f * n;
    const float* rm = rowmax + (long long)f * H;
    const T* fr = frames + (long long)f * fstride;
    // ||frame||^2 (the frame uses vector loads when its address allows) and
    // the FP32 peak from the rows' maxima
    A sqa = 0; // exact (u64) for integer frames, FP64 for float frames
    float mx = -INFINITY;
    for (int y = threadIdx.x; y < H; y += blockDim.x)
        mx = fmaxf(mx, rm[y]);
    constexpr int PV = sizeof(T) == 8 ? 2 : 4;           // pixels per frame vector load
    const bool vec = (reinterpret_cast<uintptr_t>(fr) & 15) == 0;
    for (int p = threadIdx.x * 4; p < n; p += blockDim.x * 4) {
        if (vec) {
#pragma unroll
            for (int q = 0; q < 4; q += PV) {
                T px[PV];
                if (sizeof(T) == 1)
                    *reinterpret_cast<uint32_t*>(px) = *reinterpret_cast<const uint32_t*>(fr + p + q);
                else if (sizeof(T) == 2)
                    *reinterpret_cast<uint2*>(px) = *reinterpret_cast<const uint2*>(fr + p + q);
                else
                    *reinterpret_cast<uint4*>(px) = *reinterpret_cast<const uint4*>(fr + p + q);
#pragma unroll
                for (int e = 0; e < PV; ++e)
                    sqa += mul_exact<A>(px[e], px[e]);
            }
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                sqa += mul_exact<A>(fr[p + e], fr[p + e]);
        }
    }
    const double sq = (double)block_sum(sqa, redA1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
        redF[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = redF[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i)
        mx = fmaxf(mx, redF[i]);
    const double tau = 8.0 * 5.9604644775390625e-08 * err_stages * sqrt(*ref_sq * sq) * (double)n;
    const float thr = (float)((double)mx - tau);

    A best = 0;
    int best_idx = -1;
    auto rescore = [&](int nc) {
        for (int q0 = 0; q0 < nc; q0 += kMulti) {
            const int k = nc - q0 < kMulti ? nc - q0 : kMulti;
            A v[kMulti];
            exact_corr_multi(ref, fr, W, logW, H, cand + q0, k, v, redM);
            for (int c = 0; c < k; ++c) {
                const int p = cand[q0 + c];
                if (best_idx < 0 || v[c] > best || (v[c] == best && p < best_idx)) {
                    best = v[c];
                    best_idx = p;
                }
            }
        }
    };
    // One pass over the rows whose maximum reaches thr collects every position
    // with c >= thr (the winner is chosen by exact value, then lowest index, so
    // collection order does not matter); corr rows are 16-byte aligned.
    if (threadIdx.x == 0)
        ncand = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    for (int y = threadIdx.x >> 5; y < H; y += nwarps) {
        if (!(rm[y] >= thr))
            continue;
        if ((W & 3) == 0) {
            for (int x = lane * 4; x < W; x += 128) {
                const int p = y * W + x;
                const float4 cv = *reinterpret_cast<const float4*>(c + p);
                const float e4[4] = { cv.x, cv.y, cv.z, cv.w };
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (e4[e] >= thr) {
                        const int slot = atomicAdd(&ncand, 1);
                        if (slot < kMaxCand)
                            cand[slot] = p + e;
                    }
            }
        } else { // rows not 16-byte aligned
            for (int x = lane; x < W; x += 32) {
                const int p = y * W + x;
                if (c[p] >= thr) {
                    const int slot = atomicAdd(&ncand, 1);
                    if (slot < kMaxCand)
                        cand[slot] = p;
                }
            }
        }
    }
    __syncthreads();
    const int total_cand = ncand;
    __syncthreads();
    if (total_cand <= kMaxCand) {
        rescore(total_cand);
    } else {
        // More candidates than the list holds: windows of blockDim.x
        // positions, the list re-scored and emptied whenever the next window
        // would overflow it, so every position with c >= thr is re-scored once.
        if (threadIdx.x == 0)
            ncand = 0;
        __syncthreads();
        auto flush = [&]() {
            rescore(ncand);
            __syncthreads();
            if (threadIdx.x == 0)
                ncand = 0;
            __syncthreads();
        };
        for (int base = 0; base < n; base += blockDim.x) {
            const int p = base + threadIdx.x;
            const bool hit = p < n && c[p] >= thr;
            const int wc = __syncthreads_count(hit);
            if (wc == 0)
                continue;
            if (ncand + wc > kMaxCand)
                flush();
            if (hit)
                cand[atomicAdd(&ncand, 1)] = p;
            __syncthreads();
        }
        flush();
    }
    if (threadIdx.x == 0) {
        int sx = best_idx % W, sy = best_idx / W;
        sx -= (sx < (W + 1) / 2) ? 0 : W;
        sy -= (sy < (H + 1) / 2) ? 0 : H;
        shifts[2 * f] = sx;
        shifts[2 * f + 1] = sy;
    }
}

__device__ __forceinline__ unsigned long long abs_px(unsigned long long v) { return v; }
__device__ __forceinline__ double abs_px(double v) { return fabs(v); }

// sum[y][x] += |frame[y + sy][x + sx]| where inside the frame, frames in
// order (main.cpp:293-294); the stack's frame 0 enters unshifted with its
// sign (main.cpp:266).
// Integer frames (u64 sums) are exact in any order, so the batch's frames are
// also split over gridDim.y CTAs whose partial sums are added atomically;
// float frames (f64 sums) keep one CTA per pixel block, frames in order.
template <typename T, typename A>
__global__ void __launch_bounds__(256) saa_add_kernel(A* __restrict__ sum, const T* __restrict__ frames,
                                                      long long fstride, int nframes, int first_is_frame0,
                                                      const int* __restrict__ shifts, int W, int H)
{
    extern __shared__ int2 sh[]; // this CTA's frames' shifts
    constexpr bool kExact = sizeof(A) == 8 && A(-1) > A(0); // unsigned 64-bit sum
    const int fb = (int)((long long)blockIdx.y * nframes / gridDim.y);
    const int fe = (int)((long long)(blockIdx.y + 1) * nframes / gridDim.y);
    for (int f = fb + threadIdx.x; f < fe; f += blockDim.x)
        sh[f - fb] = make_int2(shifts[2 * f], shifts[2 * f + 1]);
    __syncthreads();
    const int n = W * H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int y = p / W, x = p - y * W;
        A acc = kExact ? A(0) : sum[p];
        int f = fb;
        for (; f + 8 <= fe; f += 8) { // eight independent loads in flight, added in frame order
            A v[8];
            bool in[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int xs = x + sh[f - fb + q].x, ys = y + sh[f - fb + q].y;
                in[q] = xs >= 0 && xs < W && ys >= 0 && ys < H;
                v[q] = in[q] ? (A)frames[(long long)(f + q) * fstride + ys * W + xs] : (A)0;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (in[q])
                    acc += (first_is_frame0 && f + q == 0) ? v[q] : abs_px(v[q]);
        }
        for (; f < fe; ++f) {
            const int xs = x + sh[f - fb].x, ys = y + sh[f - fb].y;
            if (xs >= 0 && xs < W && ys >= 0 && ys < H) {
                const A v = (A)frames[(long long)f * fstride + ys * W + xs];
                acc += (first_is_frame0 && f == 0) ? v : abs_px(v);
            }
        }
        if constexpr (kExact)
            atomicAdd(reinterpret_cast<unsigned long long*>(&sum[p]), (unsigned long long)acc);
        else
            sum[p] = acc;
    }
}

template <typename T>
__global__ void sumsq_kernel(const T* __restrict__ fr, long long n, double* out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (long long p = threadIdx.x; p < n; p += blockDim.x) {
        const double v = (double)fr[p];
        s += v * v;
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0)
        *out = s;
}

cudaError_t launch_xcorr_shift(int dtype, const float* corr, const float* rowmax, const void* frames, long long fstride,
                               const void* ref, const double* ref_sq, int nframes, int first_is_frame0,
                               const Geometry& g, int* shifts, cudaStream_t st)
{
    // the correlation's FP32 error grows with the transforms' stages: log2(W H)
    // radix-2 stages, or the sum of the mixed-radix factors (each pass a sum
    // of that many terms) on the generic path
    const int logW = g.generic ? -1 : g.logW;
    double stages = g.logW + g.logH;
    if (g.generic) {
        stages = 0.0;
        for (int k = 0; k < g.pW.nf; ++k) stages += g.pW.fac[k];
        for (int k = 0; k < g.pH.nf; ++k) stages += g.pH.fac[k];
    }
    switch (dtype) {
    case 0: xcorr_shift_kernel<uint8_t><<<nframes, kShiftThreads, 0, st>>>(corr, rowmax, (const uint8_t*)frames, fstride, (const uint8_t*)ref, ref_sq, first_is_frame0, g.W, logW, g.H, stages, shifts); note_launches(1); break;
    case 1: xcorr_shift_kernel<uint16_t><<<nframes, kShiftThreads, 0, st>>>(corr, rowmax, (const uint16_t*)frames, fstride, (const uint16_t*)ref, ref_sq, first_is_frame0, g.W, logW, g.H, stages, shifts); note_launches(1); break;
    case 2: xcorr_shift_kernel<float><<<nframes, kShiftThreads, 0, st>>>(corr, rowmax, (const float*)frames, fstride, (const float*)ref, ref_sq, first_is_frame0, g.W, logW, g.H, stages, shifts); note_launches(1); break;
    default: xcorr_shift_kernel<double><<<nframes, kShiftThreads, 0, st>>>(corr, rowmax, (const double*)frames, fstride, (const double*)ref, ref_sq, first_is_frame0, g.W, logW, g.H, stages, shifts); note_launches(1); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_saa_add(int dtype, void* sum, const void* frames, long long fstride, int nframes,
                           int first_is_frame0, const int* shifts, const Geometry& g, cudaStream_t st)
{
    const int n = g.W * g.H;
    const int gx = (n + 255) / 256;
    // integer frames: frame groups of >= 32 frames, enough CTAs to fill a
    // 152-SM GPU about four deep
    constexpr int kTargetCtas = 4 * 152;
    int gy = 1;
    if (dtype <= 1) {
        gy = (kTargetCtas + gx - 1) / gx;
        gy = gy > nframes / 32 ? nframes / 32 : gy;
        gy = gy < 1 ? 1 : gy;
    }
    const dim3 grid(gx, dtype <= 1 ? gy : 1);
    const size_t shm = sizeof(int2) * (size_t)(nframes > 0 ? (nframes + grid.y - 1) / grid.y + 1 : 1);
    switch (dtype) {
    case 0: saa_add_kernel<uint8_t, unsigned long long><<<grid, 256, shm, st>>>((unsigned long long*)sum, (const uint8_t*)frames, fstride, nframes, first_is_frame0, shifts, g.W, g.H); note_launches(1); break;
    case 1: saa_add_kernel<uint16_t, unsigned long long><<<grid, 256, shm, st>>>((unsigned long long*)sum, (const uint16_t*)frames, fstride, nframes, first_is_frame0, shifts, g.W, g.H); note_launches(1); break;
    case 2: saa_add_kernel<float, double><<<grid, 256, shm, st>>>((double*)sum, (const float*)frames, fstride, nframes, first_is_frame0, shifts, g.W, g.H); note_launches(1); break;
    default: saa_add_kernel<double, double><<<grid, 256, shm, st>>>((double*)sum, (const double*)frames, fstride, nframes, first_is_frame0, shifts, g.W, g.H); note_launches(1); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_sumsq(int dtype, const void* frame, long long n, double* out, cudaStream_t st)
{
    switch (dtype) {
    case 0: sumsq_kernel<uint8_t><<<1, 1024, 0, st>>>((const uint8_t*)frame, n, out); note_launches(1); break;
    case 1: sumsq_kernel<uint16_t><<<1, 1024, 0, st>>>((const uint16_t*)frame, n, out); note_launches(1); break;
    case 2: sumsq_kernel<float><<<1, 1024, 0, st>>>((const float*)frame, n, out); note_launches(1); break;
    default: sumsq_kernel<double><<<1, 1024, 0, st>>>((const double*)frame, n, out); note_launches(1); break;
    }
    return cudaGetLastError();
}

} // namespace smip_gpu
