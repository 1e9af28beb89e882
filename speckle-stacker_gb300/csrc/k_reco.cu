// k_reco.cu -- closure-phase recovery.
//
// Replaces reconstruct_phases / calc_phase (include/phasereco.h:33-123).  The
// reference walks the spiral of NextRecoIndex (src/phasereco.cpp:17-36) and,
// for every unflagged point w, averages the unit phasors
//     phi(u) phi(v) conj(B(u,v) / |B(u,v)|)    over u + v = w,
// u and v flagged, |B| > DBL_EPSILON, v inside the bispectrum's v range.
// Each point may use phases set earlier in the same ring, so the walk is a
// strict serial chain; the parallelism is inside a point: the (d+1)^2
// candidate pairs are spread over the 1024 threads of the block and reduced
// with warp shuffles.
//
// Precision: the stored phase map and the final mean / normalisation are
// FP64; per-pair products use an FP32 mirror of the phase map and FP32
// phasors (errors ~1e-7 rad per pair, averaged).  B is read through a device
// replica of Bispectrum::get_element's index arithmetic, aliasing included.
// One CTA per job; many jobs (stacks) run in one launch.
#include "smip_dev.cuh"

namespace smip_gpu {

constexpr int kRecoThreads = 1024;

__device__ __forceinline__ int wrap_idx(int x, int y, int W, int H)
{
    return (x < 0 ? x + W : x) + (y < 0 ? y + H : y) * W;
}

// unit phasor of B as FP32 without overflow: scale by a power of two first
__device__ __forceinline__ bool unit_phasor(float2 b, float2* out)
{
    const float m = fmaxf(fabsf(b.x), fabsf(b.y));
    // |B| > DBL_EPSILON (phasereco.h:100); |B| >= m and |B| <= m*sqrt(2)
    const double eps = 2.220446049250313080847263336181640625e-16;
    if ((double)m * 1.4142135623730951 <= eps)
        return false;
    if ((double)m <= eps) {
        const double bx = b.x, by = b.y;
        if (!(sqrt(bx * bx + by * by) > eps))
            return false;
    }
    int e;
    frexpf(m, &e);
    const float sx = ldexpf(b.x, -e), sy = ldexpf(b.y, -e);
    const float r = rsqrtf(sx * sx + sy * sy);
    *out = make_float2(sx * r, sy * r);
    return true;
}

__global__ void __launch_bounds__(kRecoThreads, 1) phase_reco_kernel(const RecoJob* __restrict__ jobs)
{
    extern __shared__ unsigned int flagbits[]; // W*H bits
    __shared__ float red_r[32], red_i[32];
    __shared__ int red_n[32];
    const RecoJob J = jobs[blockIdx.x];
    const int W = J.W, H = J.H, De = J.De;
    const int nbits = W * H;
    for (int i = threadIdx.x; i < (nbits + 31) / 32; i += blockDim.x)
        flagbits[i] = 0u;
    __syncthreads();
    // seeds (phasereco.h:42-54)
    if (threadIdx.x < 5) {
        const int sx[5] = { 0, 1, 0, -1, 0 }, sy[5] = { 0, 0, 1, 0, -1 };
        const int p = wrap_idx(sx[threadIdx.x], sy[threadIdx.x], W, H);
        const double im = threadIdx.x < 3 ? 0.0 : -0.0;
        J.phases[p] = make_double2(1.0, im);
        J.phf[p] = make_float2(1.f, (float)im);
        J.cons[p] = 1.0;
        atomicOr(&flagbits[p >> 5], 1u << (p & 31));
    }
    __syncthreads();

    BispecDims d;
    const int szW = (W / 2) * 2 + 1, szH = (H / 2) * 2 + 1, szD = De + 1;
    d.sizes[0] = szW; d.sizes[1] = szH; d.sizes[2] = szD; d.sizes[3] = szD;
    d.base[0] = szW - szW / 2; d.base[1] = szH; d.base[2] = szD - szD / 2; d.base[3] = szD;
    for (int n = 0; n < 4; ++n) {
        d.mn[n] = -(d.sizes[n] / 2);
        d.mx[n] = d.sizes[n] + d.mn[n] - 1;
    }
    d.base_size = (long long)d.base[0] * d.base[1] * d.base[2] * d.base[3];
    const int pmin0 = -(W >> 1), pmin1 = -(H >> 1);
    const int pmax0 = -W / 2 + W - 1, pmax1 = -H / 2 + H - 1;
    const int nv = (De + 1) * (De + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (int q = 0; q < J.nvisits; ++q) {
        const int2 w = J.visits[q];
        if (w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1)
            continue;
        const int pw = wrap_idx(w.x, w.y, W, H);
        if (flagbits[pw >> 5] & (1u << (pw & 31)))
            continue;
        if (abs(w.x) + abs(w.y) <= 1) // phasereco.h:84-86
            continue;
        if (w.x < d.mn[0] || w.x > d.mx[0] || w.y < d.mn[1] || w.y > d.mx[1])
            continue;
        float sr = 0.f, si = 0.f;
        int cnt = 0;
        for (int t = threadIdx.x; t < nv; t += blockDim.x) {
            const int vx = -De / 2 + t % (De + 1), vy = -De / 2 + t / (De + 1);
            const int ux = w.x - vx, uy = w.y - vy;
            if (ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1)
                continue;
            const int pu = wrap_idx(ux, uy, W, H), pv = wrap_idx(vx, vy, W, H);
            if (!(flagbits[pu >> 5] & (1u << (pu & 31))) || !(flagbits[pv >> 5] & (1u << (pv & 31))))
                continue;
            int cj = 0;
            const long long off = bispec_get_offset(d, ux, uy, vx, vy, &cj);
            if (off < 0) {
                record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                continue;
            }
            float2 b = J.B[off];
            if (cj)
                b.y = -b.y;
            float2 bh;
            if (!unit_phasor(b, &bh))
                continue;
            const float2 a = J.phf[pu], c = J.phf[pv];
            const float2 pp = cmul(a, c);
            const float2 ph = cmul(pp, make_float2(bh.x, -bh.y));
            const float r = rsqrtf(ph.x * ph.x + ph.y * ph.y);
            sr += ph.x * r;
            si += ph.y * r;
            ++cnt;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) {
            red_r[warp] = sr;
            red_i[warp] = si;
            red_n[warp] = cnt;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double mr = 0.0, mi = 0.0;
            int n = 0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
                mr += (double)red_r[i];
                mi += (double)red_i[i];
                n += red_n[i];
            }
            if (n > 0) { // phasereco.h:110-122
                mr /= (double)n;
                mi /= (double)n;
                const double ab = sqrt(mr * mr + mi * mi);
                J.cons[pw] = ab;
                double2 ph = make_double2(0.0, 0.0);
                if (ab > 2.220446049250313080847263336181640625e-16)
                    ph = make_double2(mr / ab, mi / ab);
                J.phases[pw] = ph;
                J.phf[pw] = make_float2((float)ph.x, (float)ph.y);
                flagbits[pw >> 5] |= 1u << (pw & 31);
            }
        }
        __syncthreads();
    }
    // export the flag map
    for (int p = threadIdx.x; p < nbits; p += blockDim.x)
        J.flags[p] = (flagbits[p >> 5] >> (p & 31)) & 1u;
}

cudaError_t launch_phase_reco(const RecoJob* jobs_dev, int njobs, int max_W, int max_H, cudaStream_t st)
{
    const size_t smem = sizeof(unsigned int) * (((size_t)max_W * max_H + 31) / 32);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(phase_reco_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    phase_reco_kernel<<<njobs, kRecoThreads, smem, st>>>(jobs_dev);
    return cudaGetLastError();
}

} // namespace smip_gpu
