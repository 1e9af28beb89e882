// k_reco.cu -- closure-phase recovery.
//
// Replaces reconstruct_phases / calc_phase (include/phasereco.h:33-123).  The
// reference walks the spiral of NextRecoIndex (src/phasereco.cpp:17-36) and,
// for every unflagged point w, averages the unit phasors
//     phi(u) phi(v) conj(B(u,v) / |B(u,v)|)    over u + v = w,
// u and v flagged, |B| > DBL_EPSILON, v inside the bispectrum's v range.
// Each point may use phases set earlier in the same ring, so the walk is a
// strict serial chain; the parallelism is inside a point: the (d+1)^2
// candidate pairs are spread over the 512 threads of the block.
//
// Latency structure of one point: the bispectrum gathers depend only on w, not
// on the chain, so the gathers of the NEXT point are issued before the
// current point is reduced (software pipelining); the visit list is staged in
// shared memory; phases of the small v disc live in shared memory.
//
// Precision: per-pair products in FP32 from an FP32 mirror of the phase map
// (~1e-7 rad per pair); the phasor sums are compensated (float-float, ~48-bit)
// through the thread, warp and block reductions, because at low-consistency
// points the mean phasor is a large cancellation; the mean, |mean|
// (consistency) and the stored phase are FP64.  B is read through a device
// replica of Bispectrum::get_element's index arithmetic, aliasing included.
// One CTA per job; many jobs (stacks) run in one launch.
#include "smip_dev.cuh"

namespace smip_gpu {

constexpr int kRecoThreads = 512;
constexpr int kVisitChunk = 2048;
constexpr int kMaxSlots = (65 * 65 + kRecoThreads - 1) / kRecoThreads; // pair slots per thread (d <= 64)

__device__ __forceinline__ int wrap_idx(int x, int y, int W, int H)
{
    return (x < 0 ? x + W : x) + (y < 0 ? y + H : y) * W;
}

// Unit phasor of B in FP32 without overflow (scale by a power of two), and
// the reference's test |B| > DBL_EPSILON = 2^-52 (phasereco.h:100) decided
// from the binary exponent, without FP64 arithmetic.
__device__ __forceinline__ bool unit_phasor(float2 b, float2* out)
{
    const float m = fmaxf(fabsf(b.x), fabsf(b.y));
    if (!(m > 0.f))
        return false;
    int e;
    frexpf(m, &e); // m = f * 2^e, f in [0.5, 1)
    const float sx = ldexpf(b.x, -e), sy = ldexpf(b.y, -e);
    const float n2 = sx * sx + sy * sy; // |B|^2 / 4^e, in [0.25, 2)
    // |B| = 2^e sqrt(n2) with sqrt(n2) in [0.5, sqrt 2)
    if (e <= -53)
        return false;
    if (e == -52 && !(n2 > 1.f))
        return false;
    const float r = rsqrtf(n2);
    *out = make_float2(sx * r, sy * r);
    return true;
}

// float-float accumulation (Knuth two-sum).  The _rn intrinsics are never
// contracted with a product the caller passes in.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float bh, float bl)
{
    const float s = __fadd_rn(hi, bh);
    const float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    e = __fadd_rn(e, __fadd_rn(lo, bl));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// ----------------------------------------------------------------- plan
// The bispectrum side of every pair the walk can use depends only on (w, v),
// not on the chain: plan[q][t] = unit phasor of B(w_q - v_t, v_t), or
// (0, 0) when the pair never contributes (u outside the map, |B| <= eps,
// w skipped by calc_phase), or NaN where Bispectrum::get_element would throw.
// Fully parallel over (visit, v); the serial chain then only streams rows.
__global__ void __launch_bounds__(256) reco_plan_kernel(const RecoJob* __restrict__ jobs)
{
    const RecoJob J = jobs[blockIdx.y];
    const int W = J.W, H = J.H, De = J.De;
    const int nside = De + 1, nv = nside * nside;
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
    const long long total = (long long)J.nvisits * nv;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(e / nv), t = (int)(e - (long long)q * nv);
        const int2 w = J.visits[q];
        float2 out = make_float2(0.f, 0.f);
        const bool wok = !(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1) && (abs(w.x) + abs(w.y) > 1)
                         && !(w.x < d.mn[0] || w.x > d.mx[0] || w.y < d.mn[1] || w.y > d.mx[1]);
        if (wok) {
            const int vx = -De / 2 + t % nside, vy = -De / 2 + t / nside;
            const int ux = w.x - vx, uy = w.y - vy;
            if (!(ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1)) {
                int cj = 0;
                const long long off = bispec_get_offset(d, ux, uy, vx, vy, &cj);
                if (off < 0) {
                    out = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
                } else {
                    float2 b = __ldg(&J.B[off]);
                    if (cj)
                        b.y = -b.y;
                    float2 bh;
                    if (unit_phasor(b, &bh))
                        out = bh;
                }
            }
        }
        J.plan[e] = out;
    }
}

// ---------------------------------------------------------------- chain
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gmem_src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(smem_dst)), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One CTA per job walks the spiral.  For the point being reduced the plan row
// and the phases phi(u) sit in shared memory; the next point's row and phase
// gathers are already in flight (cp.async, double-buffered), so the serial
// path per point is: flag checks, two complex products, the reductions.
// kSlots = ceil((d+1)^2 / 512) pair slots per thread, fixed at compile time so
// that a small depth does not pay for the largest one's slot loop.
template <int kSlots>
__global__ void __launch_bounds__(kRecoThreads, 1) phase_chain_kernel(const RecoJob* __restrict__ jobs)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float red[3][32];
    __shared__ int red_n[32];
    __shared__ int last_pw;
    __shared__ float2 last_ph;
    const RecoJob J = jobs[blockIdx.x];
    const int W = J.W, H = J.H, De = J.De;
    const int nbits = W * H;
    const int nside = De + 1, nv = nside * nside;
    float2* rowbuf = reinterpret_cast<float2*>(smraw);          // [2][nv] plan rows
    float2* phubuf = rowbuf + 2 * nv;                            // [2][nv] phi(u) gathers
    float2* vtab = phubuf + 2 * nv;                              // [nv] phases of the v disc
    int2* vis = reinterpret_cast<int2*>(vtab + nv);              // [kVisitChunk]
    unsigned int* flagbits = reinterpret_cast<unsigned int*>(vis + kVisitChunk); // [W*H bits]
    for (int i = threadIdx.x; i < (nbits + 31) / 32; i += blockDim.x)
        flagbits[i] = 0u;
    for (int i = threadIdx.x; i < nv; i += blockDim.x)
        vtab[i] = make_float2(0.f, 0.f);
    if (threadIdx.x == 0)
        last_pw = -1;
    __syncthreads();
    if (threadIdx.x < 5) { // seeds (phasereco.h:42-54); all inside the v disc
        const int sx[5] = { 0, 1, 0, -1, 0 }, sy[5] = { 0, 0, 1, 0, -1 };
        const int p = wrap_idx(sx[threadIdx.x], sy[threadIdx.x], W, H);
        const float im = threadIdx.x < 3 ? 0.f : -0.f;
        J.phf[p] = make_float2(1.f, im);
        J.sums[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        J.cnt[p] = -1;
        vtab[(sy[threadIdx.x] + De / 2) * nside + sx[threadIdx.x] + De / 2] = make_float2(1.f, im);
        atomicOr(&flagbits[p >> 5], 1u << (p & 31));
    }
    const int pmin0 = -(W >> 1), pmin1 = -(H >> 1);
    const int pmax0 = -W / 2 + W - 1, pmax1 = -H / 2 + H - 1;
    const int szW = (W / 2) * 2 + 1, szH = (H / 2) * 2 + 1;
    const int umn0 = -(szW / 2), umx0 = szW - szW / 2 - 1, umn1 = -(szH / 2), umx1 = szH - szH / 2 - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    // This thread's pair slots t = threadIdx.x + k * kRecoThreads and their v
    // (and v's map index), computed once for the whole walk.
    int svx[kSlots], svy[kSlots], spv[kSlots];
#pragma unroll
    for (int k = 0; k < kSlots; ++k) {
        const int t = threadIdx.x + k * kRecoThreads;
        svx[k] = -De / 2 + t % nside;
        svy[k] = -De / 2 + t / nside;
        spv[k] = t < nv ? wrap_idx(svx[k], svy[k], W, H) : 0;
    }

    // each thread copies its own slots and later reads only what it copied
    auto prefetch = [&](int q, int2 w, int buf) {
        const float2* row = J.plan + (long long)q * nv;
#pragma unroll
        for (int k = 0; k < kSlots; ++k) {
            const int t = threadIdx.x + k * kRecoThreads;
            if (t < nv) {
                cp_async8(&rowbuf[buf * nv + t], &row[t]);
                const int ux = w.x - svx[k], uy = w.y - svy[k];
                if (!(ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1))
                    cp_async8(&phubuf[buf * nv + t], &J.phf[wrap_idx(ux, uy, W, H)]);
            }
        }
        cp_async_commit();
    };

    __syncthreads();
    int2 wcur = J.visits[0];
    prefetch(0, wcur, 0);
    for (int q0 = 0; q0 < J.nvisits; q0 += kVisitChunk) {
        const int nq = min(kVisitChunk, J.nvisits - q0);
        __syncthreads();
        for (int i = threadIdx.x; i < nq; i += blockDim.x)
            vis[i] = J.visits[q0 + i];
        __syncthreads();
        for (int qi = 0; qi < nq; ++qi) {
            const int q = q0 + qi;
            const int buf = q & 1;
            // this point's copies (issued one point ago) land; only then is the
            // other buffer free for the next point's copies
            cp_async_wait_all();
            int2 wn = make_int2(0, 0);
            if (q + 1 < J.nvisits) {
                wn = qi + 1 < nq ? vis[qi + 1] : J.visits[q + 1];
                prefetch(q + 1, wn, buf ^ 1);
            }
            const int2 w = wcur;
            bool run = !(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1);
            const int pw = run ? wrap_idx(w.x, w.y, W, H) : 0;
            run = run && !(flagbits[pw >> 5] & (1u << (pw & 31)));
            run = run && (abs(w.x) + abs(w.y) > 1);                                   // phasereco.h:84
            run = run && !(w.x < umn0 || w.x > umx0 || w.y < umn1 || w.y > umx1);
            if (run) {
                const int lpw = last_pw;
                const float2 lph = last_ph;
                float sr = 0.f, si = 0.f;
                int cnt = 0;
#pragma unroll
                for (int k = 0; k < kSlots; ++k) {
                    const int t = threadIdx.x + k * kRecoThreads;
                    if (t >= nv)
                        continue;
                    const float2 bh = rowbuf[buf * nv + t];
                    if (bh.x == 0.f && bh.y == 0.f)
                        continue;
                    const int pu = wrap_idx(w.x - svx[k], w.y - svy[k], W, H), pv = spv[k];
                    if (!(flagbits[pu >> 5] & (1u << (pu & 31))) || !(flagbits[pv >> 5] & (1u << (pv & 31))))
                        continue;
                    if (isnan(bh.x)) {
                        record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                        continue;
                    }
                    const float2 phu = pu == lpw ? lph : phubuf[buf * nv + t];
                    const float2 ph = cmul(cmul(phu, vtab[t]), make_float2(bh.x, -bh.y));
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
                    red[0][warp] = sr;
                    red[1][warp] = si;
                    red_n[warp] = cnt;
                }
                __syncthreads();
                if (warp == 0) {
                    // float-float across warps: the mean phasor can be a large cancellation
                    constexpr int nw = kRecoThreads / 32;
                    float rh = lane < nw ? red[0][lane] : 0.f, rl = 0.f;
                    float ih = lane < nw ? red[1][lane] : 0.f, il = 0.f;
                    cnt = lane < nw ? red_n[lane] : 0;
#pragma unroll
                    for (int o = nw / 2; o > 0; o >>= 1) {
                        const float a = __shfl_xor_sync(0xffffffffu, rh, o), b = __shfl_xor_sync(0xffffffffu, rl, o);
                        const float c = __shfl_xor_sync(0xffffffffu, ih, o), e = __shfl_xor_sync(0xffffffffu, il, o);
                        ff_add(rh, rl, a, b);
                        ff_add(ih, il, c, e);
                        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
                    }
                    if (lane == 0 && cnt > 0) {
                        // FP32 phase for the chain; FP64 values are formed after the walk
                        const float s2 = rh * rh + ih * ih;
                        const float lim = 2.220446049250313e-16f * (float)cnt;
                        float2 pf = make_float2(0.f, 0.f);
                        if (s2 > lim * lim) {
                            const float r = rsqrtf(s2);
                            pf = make_float2(rh * r, ih * r);
                        }
                        J.phf[pw] = pf;
                        J.sums[pw] = make_float4(rh, rl, ih, il);
                        J.cnt[pw] = cnt;
                        if (abs(w.x) <= De / 2 && abs(w.y) <= De / 2)
                            vtab[(w.y + De / 2) * nside + w.x + De / 2] = pf;
                        flagbits[pw >> 5] |= 1u << (pw & 31);
                        last_pw = pw;
                        last_ph = pf;
                    }
                }
                __syncthreads();
            }
            wcur = wn;
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // FP64 mean, consistency and phase of every point (phasereco.h:110-122),
    // and the flag map
    for (int p = threadIdx.x; p < nbits; p += blockDim.x) {
        const unsigned f = (flagbits[p >> 5] >> (p & 31)) & 1u;
        J.flags[p] = f;
        if (!f)
            continue;
        const int n = J.cnt[p];
        if (n < 0) { // seed
            J.phases[p] = make_double2(1.0, J.phf[p].y);
            J.cons[p] = 1.0;
            continue;
        }
        const float4 s = J.sums[p];
        const double mr = ((double)s.x + (double)s.y) / (double)n;
        const double mi = ((double)s.z + (double)s.w) / (double)n;
        const double ab = sqrt(mr * mr + mi * mi);
        J.cons[p] = ab;
        J.phases[p] = ab > 2.220446049250313080847263336181640625e-16 ? make_double2(mr / ab, mi / ab)
                                                                      : make_double2(0.0, 0.0);
    }
}

// Runs the device get_element index replica on a list of 4-index tuples.
__global__ void bispec_offset_probe_kernel(BispecDims d, const int4* __restrict__ idx, long long n,
                                           long long* __restrict__ off, int* __restrict__ conj)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int4 i = idx[q];
        int cj = 0;
        off[q] = bispec_get_offset(d, i.x, i.y, i.z, i.w, &cj);
        conj[q] = off[q] < 0 ? 0 : cj;
    }
}

cudaError_t launch_offset_probe(const Geometry& g, const int* idx, long long n, long long* off, int* conj,
                                cudaStream_t st)
{
    BispecDims d;
    const int szW = (g.W / 2) * 2 + 1, szH = (g.H / 2) * 2 + 1, szD = g.De + 1;
    d.sizes[0] = szW; d.sizes[1] = szH; d.sizes[2] = szD; d.sizes[3] = szD;
    d.base[0] = szW - szW / 2; d.base[1] = szH; d.base[2] = szD - szD / 2; d.base[3] = szD;
    for (int k = 0; k < 4; ++k) {
        d.mn[k] = -(d.sizes[k] / 2);
        d.mx[k] = d.sizes[k] + d.mn[k] - 1;
    }
    d.base_size = (long long)d.base[0] * d.base[1] * d.base[2] * d.base[3];
    bispec_offset_probe_kernel<<<256, 256, 0, st>>>(d, reinterpret_cast<const int4*>(idx), n, off, conj); note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_phase_reco(const RecoJob* jobs_dev, int njobs, int max_W, int max_H, int max_De, cudaStream_t st)
{
    const int nv = (max_De + 1) * (max_De + 1);
    reco_plan_kernel<<<dim3(1024, njobs), 256, 0, st>>>(jobs_dev);
    note_launches(1);
    const size_t smem = sizeof(float2) * 5 * nv + sizeof(int2) * kVisitChunk
                        + sizeof(unsigned int) * (((size_t)max_W * max_H + 31) / 32);
    const int slots = (nv + kRecoThreads - 1) / kRecoThreads;
    auto launch = [&](auto kern) -> cudaError_t {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess)
                return e;
        }
        kern<<<njobs, kRecoThreads, smem, st>>>(jobs_dev);
        note_launches(1);
        return cudaGetLastError();
    };
    static_assert(kMaxSlots == 9, "slot instantiations");
    switch (slots) {
    case 1: return launch(phase_chain_kernel<1>);
    case 2: return launch(phase_chain_kernel<2>);
    case 3: return launch(phase_chain_kernel<3>);
    case 4: return launch(phase_chain_kernel<4>);
    case 5: return launch(phase_chain_kernel<5>);
    case 6: return launch(phase_chain_kernel<6>);
    case 7: return launch(phase_chain_kernel<7>);
    case 8: return launch(phase_chain_kernel<8>);
    default: return launch(phase_chain_kernel<9>);
    }
}

} // namespace smip_gpu
