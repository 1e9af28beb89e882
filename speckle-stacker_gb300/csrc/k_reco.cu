// k_reco.cu -- closure-phase recovery.
//
// Replaces reconstruct_phases / calc_phase (include/phasereco.h:33-123).  The
// reference walks the spiral of NextRecoIndex (src/phasereco.cpp:17-36) and,
// for every unflagged point w, averages the unit phasors
//     phi(u) phi(v) conj(B(u,v) / |B(u,v)|)    over u + v = w,
// u and v flagged, |B| > DBL_EPSILON, v inside the bispectrum's v range.
// Each point may use phases set earlier in the same ring, so the walk is a
// serial chain.  Most of a point's pairs, though, read phases that were final
// long before: a pair is "recent" only when u or v was visited within the
// kRecoLag visits before w (the arc of the ring just behind w).  The walk is
// therefore split:
//   - summing warps form, for visit q, the sum over its non-recent pairs as
//     soon as the walk has passed q - kRecoLag, eight pair slots per lane at a
//     time so that the plan, flag and phase gathers overlap;
//   - one serial warp runs the visits in order and adds only the recent pairs (a list
//     of at most kRecentMax per visit, prefetched with the plan phasors) to
//     that share, then sets the point's phase and flag.
// Which pairs are recent depends only on the visit list (per point: its visit
// indices), so it is computed in parallel before the walk.
// Depths below kClusterDepth walk in one CTA (phase_pipe_kernel); deeper
// bispectra, whose (d+1)^2 pairs per visit one CTA's summing warps cannot
// keep up with, walk in a thread-block cluster (phase_cluster_kernel).
//
// Precision: per-pair products in FP32 from an FP32 mirror of the phase map
// (~1e-7 rad per pair); the non-recent share is summed in FP32 per lane and in
// float-float over the lanes, and the recent pairs are added to it in
// float-float, because at low-consistency points the mean phasor is a large
// cancellation; the mean, |mean| (consistency) and the stored phase are FP64.
// B is read through a device replica of Bispectrum::get_element's index
// arithmetic, aliasing included.
#include <type_traits>

#include "smip_dev.cuh"

namespace smip_gpu {

constexpr int kRecoThreads = 512;

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

// ------------------------------------------------------ pipelined walk
// A visit's pairs split by when their phases became final.  A pair (u, v)
// of visit q is "recent" when u or v was visited within the kRecoLag visits
// before q (visit lists per point: pvis); every other pair only reads phases
// and flags that no visit in [q - kRecoLag, q) can change, so its share of
// the sum can be formed as soon as the walk has passed q - kRecoLag.  The
// serial part of a visit is then the few recent pairs (the arc of the current
// ring just behind w) instead of all (d+1)^2.
__device__ __forceinline__ bool visited_in_lag(int4 pv, int q)
{
    if (pv.w > 3) // more visits than recorded: treat as recent
        return true;
    const int lo = q - kRecoLag;
    return (pv.x >= 0 && pv.x >= lo && pv.x < q) || (pv.y >= 0 && pv.y >= lo && pv.y < q)
           || (pv.z >= 0 && pv.z >= lo && pv.z < q);
}

__global__ void __launch_bounds__(256) reco_recent_kernel(const RecoJob* __restrict__ jobs)
{
    const RecoJob J = jobs[blockIdx.y];
    const int W = J.W, H = J.H, De = J.De;
    const int nside = De + 1, nv = nside * nside, nwords = (nv + 31) / 32;
    const int pmin0 = -(W >> 1), pmin1 = -(H >> 1);
    const int pmax0 = -W / 2 + W - 1, pmax1 = -H / 2 + H - 1;
    const long long total = (long long)J.nvisits * nwords;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(e / nwords), wd = (int)(e - (long long)q * nwords);
        const int2 w = J.visits[q];
        unsigned bits = 0u;
        if (!(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1)) {
            for (int b = 0; b < 32; ++b) {
                const int t = wd * 32 + b;
                if (t >= nv)
                    break;
                const int vx = -De / 2 + t % nside, vy = -De / 2 + t / nside;
                const int ux = w.x - vx, uy = w.y - vy;
                if (ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1)
                    continue;
                if (visited_in_lag(J.pvis[wrap_idx(ux, uy, W, H)], q) || visited_in_lag(J.pvis[wrap_idx(vx, vy, W, H)], q))
                    bits |= 1u << b;
            }
        }
        J.rbits[e] = bits;
    }
}

// One warp per visit: the recent pair slots in increasing order, or -1 when
// there are more than kRecentMax (the serial warp then takes every pair).
__global__ void __launch_bounds__(256) reco_rlist_kernel(const RecoJob* __restrict__ jobs)
{
    const RecoJob J = jobs[blockIdx.y];
    const int nv = (J.De + 1) * (J.De + 1), nwords = (nv + 31) / 32;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int q = gw; q < J.nvisits; q += nw) {
        const unsigned* rb = J.rbits + (long long)q * nwords;
        int base = 0;
        for (int w0 = 0; w0 < nwords; w0 += 32) {
            const unsigned bits = w0 + lane < nwords ? rb[w0 + lane] : 0u;
            const int c = __popc(bits);
            int incl = c; // inclusive prefix over the lanes
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o)
                    incl += y;
            }
            int pos = base + incl - c;
            unsigned b = bits;
            while (b) {
                const int k = __ffs(b) - 1;
                b &= b - 1;
                if (pos < kRecentMax)
                    J.rlist[(long long)q * kRecentMax + pos] = (unsigned short)((w0 + lane) * 32 + k);
                ++pos;
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0)
            J.rcount[q] = base > kRecentMax ? -1 : base;
    }
}

// The walk, one thread-block cluster per job.  Warp 0 of the cluster's rank-0
// CTA runs the visits in order: for visit q it waits for the share of the
// non-recent pairs, adds the recent pairs (or all pairs when the list
// overflowed), forms the phase and advances `progress`.  The warps of the
// other CTAs form the non-recent shares of visits q = g (mod number of such
// warps), each once progress >= q - kRecoLag, and store them into a ring of
// kRing slots in rank 0's shared memory.  A visit's share is split into up to
// kMaxParts parts over ranges of its pair slots, summed by different warps
// (only the kRecoLag visits ahead of the walk can be summed at any time, so
// a visit's latency, not the warp count, sets the rate), and the serial warp
// adds the parts in part order (distributed shared memory: st.async stores that complete
// the slot's mbarrier, on which the serial warp waits locally).  `progress`
// is published with a release at cluster scope, so the summing warps, after
// their acquire, read the phases and flags the walk set from the phase map in
// global memory, where an unflagged point holds NaN.  Rank 0 keeps its SM
// for the serial warp (summing warps beside it take its issue slots: 3.4k
// against 2.3k cycles per visit at 256 x 256, d = 32); a cluster of one CTA
// (where the GPU cannot place more) sums on its other warps.  Every wait is
// bounded; on a timeout the walk stops and the error is recorded.
constexpr int kRing = 64;
constexpr int kPhaseCache = 2048;
// CTAs per job (cluster size) from depth kClusterDepth on, fewer where the GPU
// cannot place 8.  Below it phase_pipe_kernel walks in one CTA: its summing
// warps keep up with the serial warp (256 x 256, d = 32, R = 128: 58.0 ms in
// one CTA, 59.4 ms in a cluster), and a cluster would hold 8 SMs instead of 1
// while it walks, which other jobs sharing the GPU need.
constexpr int kWalkCtas = 8;
constexpr int kClusterDepth = 40;
constexpr uint32_t kShareBytes = sizeof(float4) + sizeof(int); // one part's st.async payload
constexpr int kMaxParts = 6;
// static + the largest dynamic shared memory (1024 x 1024 flags, d = 64) fit a CTA's 227 KB
static_assert(kRing * kMaxParts * (sizeof(float4) + sizeof(int)) + kRing * 8 + kPhaseCache * (sizeof(int) + sizeof(float2))
                      + 64 + (sizeof(float2) + sizeof(int2)) * 65 * 65 + sizeof(unsigned) * (kMaxSide * kMaxSide / 32)
                  <= 227 * 1024,
              "walk shared memory");

// parts per visit share: about 16 words of pair slots (512 slots) each
__host__ __device__ __forceinline__ int share_parts(int nwords)
{
    const int p = nwords / 16;
    return p < 1 ? 1 : (p > kMaxParts ? kMaxParts : p);
}

// CTA-scope acquire load / release store on shared memory: they order the
// accesses after (before) them without waiting for this thread's other
// outstanding loads, as a full fence would.
__device__ __forceinline__ void st_release_cta(int* p, int v)
{
    asm volatile("st.release.cta.shared.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
static_assert(kRing > kRecoLag + 1, "ring slots outlive the lag");
constexpr unsigned long long kRecoWaitNs = 2000000000ull;

__device__ __forceinline__ bool unflagged(float2 ph) { return isnan(ph.x); }

__global__ void __launch_bounds__(kRecoThreads, 1) phase_cluster_kernel(const RecoJob* __restrict__ jobs)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float4 ring_s[kRing][kMaxParts];
    __shared__ int ring_n[kRing][kMaxParts];
    __shared__ __align__(8) uint64_t ring_bar[kRing]; // slot q % kRing: visit q's share has landed
    __shared__ int progress;
    __shared__ int abort_walk;
    __shared__ int pc_key[kPhaseCache];   // serial warp: phases it set, by point
    __shared__ float2 pc_val[kPhaseCache];
    const uint32_t rank = cluster_rank(), ncta = cluster_size();
    const RecoJob J = jobs[blockIdx.x / ncta];
    const int W = J.W, H = J.H, De = J.De;
    const int nbits = W * H;
    const int nside = De + 1, nv = nside * nside, nwords = (nv + 31) / 32;
    const int nparts = share_parts(nwords);
    float2* vtab = reinterpret_cast<float2*>(smraw);                        // [nv] phases of the v disc (rank 0)
    int2* slot_v = reinterpret_cast<int2*>(vtab + nv);                      // [nv] (vx | vy << 16, map index of v)
    unsigned int* flagbits = reinterpret_cast<unsigned int*>(slot_v + nv);  // [W*H bits] (rank 0)
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        const int vx = -De / 2 + i % nside, vy = -De / 2 + i / nside;
        slot_v[i] = make_int2((int)(((unsigned)vx & 0xffffu) | ((unsigned)vy << 16)), wrap_idx(vx, vy, W, H));
    }
    if (rank == 0) {
        for (int i = threadIdx.x; i < (nbits + 31) / 32; i += blockDim.x)
            flagbits[i] = 0u;
        for (int i = threadIdx.x; i < nv; i += blockDim.x)
            vtab[i] = make_float2(0.f, 0.f);
        if (threadIdx.x == 0) {
            progress = 0;
            abort_walk = 0;
            for (int i = 0; i < kRing; ++i) // one arrival per phase: the serial warp's expect_tx
                mbar_init(&ring_bar[i], 1);
            fence_mbar_init();
        }
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
    }
    cluster_sync_all(); // rank 0's ring, progress and the seeds are set
    const int pmin0 = -(W >> 1), pmin1 = -(H >> 1);
    const int pmax0 = -W / 2 + W - 1, pmax1 = -H / 2 + H - 1;
    const int szW = (W / 2) * 2 + 1, szH = (H / 2) * 2 + 1;
    const int umn0 = -(szW / 2), umx0 = szW - szW / 2 - 1, umn1 = -(szH / 2), umx1 = szH - szH / 2 - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t a_abort = dsmem_addr(&abort_walk, 0);
    const uint32_t a_progress = dsmem_addr(&progress, 0);

    auto flag = [&](int p) { return ((flagbits[p >> 5] >> (p & 31)) & 1u) != 0u; };
    // bounded wait on a condition; false on a timeout or when another warp
    // of the cluster gave up (then the walk stops)
    auto wait_until = [&](auto cond) {
        if (cond())
            return true;
        const unsigned long long t0 = globaltimer_ns();
        for (;;) {
            for (int i = 0; i < 64; ++i)
                if (cond())
                    return true;
            if (dsmem_ld_relaxed(a_abort))
                return false;
            if (globaltimer_ns() - t0 > kRecoWaitNs) {
                record_error(J.err, SMIP_DEV_ERR_TIMEOUT);
                dsmem_st_relaxed(a_abort, 1);
                return false;
            }
        }
    };

    // Pairs of visit q, eight slots per lane at a time, so that the plan and
    // phase gathers overlap.  skip_recent leaves the recent pairs out (the
    // serial warp takes them).  LOCAL: the serial warp's view (flags and v
    // phases in rank 0's shared memory, u phases from `phase`); otherwise
    // flags and both phases from the phase map in global memory (NaN: no
    // phase yet).
    // Words [wb, we) of the visit's pair slots.
    auto sum_pairs = [&](int q, int2 w, bool skip_recent, auto local, auto phase, int wb, int we, float& sr, float& si,
                         int& cnt) {
        constexpr bool LOCAL = decltype(local)::value;
        constexpr int kB = 8;
        const unsigned* rb = J.rbits + (long long)q * nwords;
        const float2* prow = J.plan + (long long)q * nv;
        for (int i0 = wb; i0 < we; i0 += kB) {
            float2 bh[kB], ph[kB], pvv[kB];
            bool use[kB];
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                const int t = lane + 32 * (i0 + k);
                use[k] = i0 + k < we && t < nv;
                // slot t's bit is bit `lane` of word i0 + k
                if (skip_recent)
                    use[k] = use[k] && !((rb[i0 + k] >> lane) & 1u);
                bh[k] = use[k] ? prow[t] : make_float2(0.f, 0.f);
                if (use[k]) { // the flags and phase gathers do not wait for the plan
                    const int2 sv = slot_v[t];
                    const int vx = (int)(short)(sv.x & 0xffff), vy = sv.x >> 16;
                    const int ux = w.x - vx, uy = w.y - vy;
                    const bool inu = !(ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1);
                    const int pu = inu ? wrap_idx(ux, uy, W, H) : 0, pv = sv.y;
                    if constexpr (LOCAL) {
                        use[k] = inu && flag(pu) && flag(pv);
                        ph[k] = use[k] ? phase(pu) : make_float2(0.f, 0.f);
                        pvv[k] = vtab[t];
                    } else {
                        ph[k] = inu ? J.phf[pu] : make_float2(0.f, 0.f);
                        pvv[k] = J.phf[pv];
                        use[k] = inu;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                if constexpr (!LOCAL)
                    use[k] = use[k] && !unflagged(ph[k]) && !unflagged(pvv[k]);
                if (!use[k] || (bh[k].x == 0.f && bh[k].y == 0.f)) // the plan's zero: never contributes
                    continue;
                if (isnan(bh[k].x)) {
                    record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                    continue;
                }
                const float2 p = cmul(cmul(ph[k], pvv[k]), make_float2(bh[k].x, -bh[k].y));
                const float r = rsqrtf(p.x * p.x + p.y * p.y);
                sr += p.x * r;
                si += p.y * r;
                ++cnt;
            }
        }
    };
    using Local = std::true_type;
    using Global = std::false_type;

    if (rank == 0 && warp == 0) {
        // ------------------------------------------------ serial warp
        // Visit data that does not depend on the walk is loaded ahead: the
        // visit, its recent-pair count and slots two visits ahead, their plan
        // phasors one visit ahead.  Phases the walk just set come from a
        // shared-memory cache keyed by point (a miss reads the phase map).
        for (int i = lane; i < kPhaseCache; i += 32)
            pc_key[i] = -1;
        __syncwarp();
        struct Ahead {
            int2 w;
            int rc, ta, tb;
            float2 ba, bb;
        };
        // the list slots are loaded without waiting for the count (a visit's
        // kRecentMax entries are always allocated) and masked one visit later
        auto load_meta = [&](int q, Ahead& a) {
            if (q >= J.nvisits)
                return;
            a.w = J.visits[q];
            a.rc = J.rcount[q];
            const unsigned short* rl = J.rlist + (long long)q * kRecentMax;
            a.ta = rl[lane];
            a.tb = rl[lane + 32];
        };
        auto load_plan = [&](int q, Ahead& a) {
            if (q >= J.nvisits)
                return;
            a.ta = lane < a.rc ? a.ta : -1;
            a.tb = lane + 32 < a.rc ? a.tb : -1;
            const float2* prow = J.plan + (long long)q * nv;
            a.ba = a.ta >= 0 ? prow[a.ta] : make_float2(0.f, 0.f);
            a.bb = a.tb >= 0 ? prow[a.tb] : make_float2(0.f, 0.f);
        };
        // every slot expects its first visit's share (visits 0 .. kRing-1)
        if (lane == 0)
            for (int i = 0; i < kRing; ++i)
                mbar_arrive_expect_tx(&ring_bar[i], kShareBytes * nparts);
        Ahead c0 {}, c1 {}, c2 {};
        load_meta(0, c0);
        load_plan(0, c0);
        load_meta(1, c1);
        auto phase_of = [&](int p) {
            const int h = p & (kPhaseCache - 1);
            return pc_key[h] == p ? pc_val[h] : J.phf[p];
        };
        auto term_s = [&](int t, float2 bh, int2 w, float& sr, float& si, int& cnt) {
            if (bh.x == 0.f && bh.y == 0.f)
                return;
            const int2 sv = slot_v[t];
            const int vx = (int)(short)(sv.x & 0xffff), vy = sv.x >> 16;
            const int pu = wrap_idx(w.x - vx, w.y - vy, W, H), pv = sv.y;
            if (!flag(pu) || !flag(pv))
                return;
            if (isnan(bh.x)) {
                record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                return;
            }
            const float2 ph = cmul(cmul(phase_of(pu), vtab[t]), make_float2(bh.x, -bh.y));
            const float r = rsqrtf(ph.x * ph.x + ph.y * ph.y);
            sr += ph.x * r;
            si += ph.y * r;
            ++cnt;
        };
        for (int q = 0; q < J.nvisits; ++q) {
            load_plan(q + 1, c1); // its slots were loaded one visit ago
            load_meta(q + 2, c2);
            const int2 w = c0.w;
            bool run = !(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1);
            const int pw = run ? wrap_idx(w.x, w.y, W, H) : 0;
            run = run && !flag(pw);
            run = run && (abs(w.x) + abs(w.y) > 1);                                   // phasereco.h:84
            run = run && !(w.x < umn0 || w.x > umx0 || w.y < umn1 || w.y > umx1);
            // every visit's share lands (the summing warps do not know which
            // visits run).  The slot is re-armed for visit q + kRing at once:
            // its next share cannot land before progress passes q + kRing -
            // kRecoLag, and an arrive here, before this visit's global stores,
            // does not wait for them (an arrive is a release)
            const int slot = q % kRing;
            if (!__all_sync(0xffffffffu,
                            wait_until([&] { return mbar_try_wait(&ring_bar[slot], (uint32_t)(q / kRing) & 1u); }) ? 1 : 0))
                break;
            if (lane == 0 && q + kRing < J.nvisits)
                mbar_arrive_expect_tx(&ring_bar[slot], kShareBytes * nparts);
            if (run) {
                float sr = 0.f, si = 0.f;
                int cnt = 0;
                if (c0.rc >= 0) {
                    if (c0.ta >= 0)
                        term_s(c0.ta, c0.ba, w, sr, si, cnt);
                    if (c0.tb >= 0)
                        term_s(c0.tb, c0.bb, w, sr, si, cnt);
                } else {
                    sum_pairs(q, w, false, Local {}, phase_of, 0, nwords, sr, si, cnt);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    sr += __shfl_xor_sync(0xffffffffu, sr, o);
                    si += __shfl_xor_sync(0xffffffffu, si, o);
                    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
                }
                if (lane == 0) {
                    // float-float: the non-recent share's parts in order, plus the recent one
                    const float4 o4 = ring_s[slot][0];
                    float rh = o4.x, rl = o4.y, ih = o4.z, il = o4.w;
                    cnt += ring_n[slot][0];
                    for (int pp = 1; pp < nparts; ++pp) {
                        const float4 op = ring_s[slot][pp];
                        ff_add(rh, rl, op.x, op.y);
                        ff_add(ih, il, op.z, op.w);
                        cnt += ring_n[slot][pp];
                    }
                    ff_add(rh, rl, sr, 0.f);
                    ff_add(ih, il, si, 0.f);
                    if (cnt > 0) {
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
                        pc_val[pw & (kPhaseCache - 1)] = pf;
                        pc_key[pw & (kPhaseCache - 1)] = pw;
                        flagbits[pw >> 5] |= 1u << (pw & 31);
                    }
                }
                __syncwarp();
            }
            // publish progress every 16 visits (a release store at cluster
            // scope, which waits for this thread's stores to the phase map
            // to reach every CTA; the lag leaves the slack)
            if (((q & 15) == 15 || q + 1 == J.nvisits) && lane == 0)
                dsmem_st_release(a_progress, q + 1);
            __syncwarp();
            c0 = c1;
            c1 = c2;
        }
    } else {
        // ------------------------------------------- non-recent shares
        const int nsum = ncta > 1 ? (int)(ncta - 1) * (kRecoThreads / 32) : kRecoThreads / 32 - 1;
        const int g = ncta > 1 ? (int)(rank - 1) * (kRecoThreads / 32) + warp : warp - 1;
        const long long nitems = (long long)J.nvisits * nparts; // (visit, part), visits in order
        for (long long it = (ncta > 1 && rank == 0) ? nitems : g; it < nitems; it += nsum) {
            const int q = (int)(it / nparts), part = (int)(it - (long long)q * nparts);
            if (!__all_sync(0xffffffffu, wait_until([&] { return dsmem_ld_acquire(a_progress) >= q - kRecoLag; }) ? 1 : 0))
                break;
            const int2 w = J.visits[q];
            const int rc = J.rcount[q];
            float sr = 0.f, si = 0.f;
            int cnt = 0;
            const bool inmap = !(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1);
            if (rc >= 0 && inmap)
                sum_pairs(q, w, true, Global {}, 0, (int)((long long)part * nwords / nparts),
                          (int)((long long)(part + 1) * nwords / nparts), sr, si, cnt);
            // float-float over the lanes, lane 0's order
            float rh = sr, rl = 0.f, ih = si, il = 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float a = __shfl_xor_sync(0xffffffffu, rh, o), b = __shfl_xor_sync(0xffffffffu, rl, o);
                const float c = __shfl_xor_sync(0xffffffffu, ih, o), e = __shfl_xor_sync(0xffffffffu, il, o);
                ff_add(rh, rl, a, b);
                ff_add(ih, il, c, e);
                cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            }
            if (lane == 0) {
                const int slot = q % kRing;
                const uint32_t bar = dsmem_addr(&ring_bar[slot], 0);
                dsmem_st_async_f4(dsmem_addr(&ring_s[slot][part], 0), make_float4(rh, rl, ih, il), bar);
                dsmem_st_async_i(dsmem_addr(&ring_n[slot][part], 0), cnt, bar);
            }
            __syncwarp();
        }
    }
    cluster_sync_all(); // no CTA reads or writes rank 0's shared memory after this
    if (rank != 0)
        return;
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

// The walk in one CTA per job (depths below kClusterDepth).  Warp 0 runs the visits in order: for visit q it
// waits for the share of the non-recent pairs, adds the recent pairs (or all
// pairs when the list overflowed), forms the phase and advances `progress`.
// Warps 1..15 form the non-recent shares of visits q = warp-1 (mod 15), each
// once progress >= q - kRecoLag, into a ring of kRing slots.  Every wait is
// bounded; on a timeout the walk stops and the error is recorded.

// CTA-scope acquire load / release store on shared memory: they order the
// accesses after (before) them without waiting for this thread's other
// outstanding loads, as a full fence would.
__device__ __forceinline__ int ld_acquire_cta(const int* p)
{
    int v;
    asm volatile("ld.acquire.cta.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}

__global__ void __launch_bounds__(kRecoThreads, 1) phase_pipe_kernel(const RecoJob* __restrict__ jobs)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float4 ring_s[kRing];
    __shared__ int ring_n[kRing];
    __shared__ int ring_tag[kRing];
    __shared__ int progress;
    __shared__ int abort_walk;
    __shared__ int pc_key[kPhaseCache];   // serial warp: phases it set, by point
    __shared__ float2 pc_val[kPhaseCache];
    const RecoJob J = jobs[blockIdx.x];
    const int W = J.W, H = J.H, De = J.De;
    const int nbits = W * H;
    const int nside = De + 1, nv = nside * nside, nwords = (nv + 31) / 32;
    float2* vtab = reinterpret_cast<float2*>(smraw);                        // [nv] phases of the v disc
    int2* slot_v = reinterpret_cast<int2*>(vtab + nv);                      // [nv] (vx | vy << 16, map index of v)
    unsigned int* flagbits = reinterpret_cast<unsigned int*>(slot_v + nv);  // [W*H bits]
    for (int i = threadIdx.x; i < (nbits + 31) / 32; i += blockDim.x)
        flagbits[i] = 0u;
    for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        vtab[i] = make_float2(0.f, 0.f);
        const int vx = -De / 2 + i % nside, vy = -De / 2 + i / nside;
        slot_v[i] = make_int2((int)(((unsigned)vx & 0xffffu) | ((unsigned)vy << 16)), wrap_idx(vx, vy, W, H));
    }
    for (int i = threadIdx.x; i < kRing; i += blockDim.x)
        ring_tag[i] = -1;
    if (threadIdx.x == 0) {
        progress = 0;
        abort_walk = 0;
    }
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
    __syncthreads();
    const int pmin0 = -(W >> 1), pmin1 = -(H >> 1);
    const int pmax0 = -W / 2 + W - 1, pmax1 = -H / 2 + H - 1;
    const int szW = (W / 2) * 2 + 1, szH = (H / 2) * 2 + 1;
    const int umn0 = -(szW / 2), umx0 = szW - szW / 2 - 1, umn1 = -(szH / 2), umx1 = szH - szH / 2 - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    volatile int* vabort = &abort_walk;

    auto flag = [&](int p) { return ((flagbits[p >> 5] >> (p & 31)) & 1u) != 0u; };
    // bounded wait on a shared-memory condition; false on a timeout (then the walk stops)
    auto wait_until = [&](auto cond) {
        if (cond())
            return true;
        const unsigned long long t0 = globaltimer_ns();
        for (;;) {
            for (int i = 0; i < 64; ++i)
                if (cond())
                    return true;
            if (*vabort)
                return false;
            if (globaltimer_ns() - t0 > kRecoWaitNs) {
                record_error(J.err, SMIP_DEV_ERR_TIMEOUT);
                *vabort = 1;
                return false;
            }
        }
    };

    // Pairs of visit q, eight slots per lane at a time, so that the plan,
    // flag and phase gathers overlap; skip_recent leaves the recent pairs
    // out (the serial warp takes them); phase reads the phase map.
    auto sum_pairs = [&](int q, int2 w, bool skip_recent, auto phase, float& sr, float& si, int& cnt) {
        constexpr int kB = 8;
        const unsigned* rb = J.rbits + (long long)q * nwords;
        const float2* prow = J.plan + (long long)q * nv;
        for (int i0 = 0; i0 < nwords; i0 += kB) {
            float2 bh[kB], ph[kB];
            int tt[kB];
            bool use[kB];
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                const int t = lane + 32 * (i0 + k);
                tt[k] = t;
                use[k] = i0 + k < nwords && t < nv;
                // slot t's bit is bit `lane` of word i0 + k
                if (skip_recent)
                    use[k] = use[k] && !((rb[i0 + k] >> lane) & 1u);
                bh[k] = use[k] ? prow[t] : make_float2(0.f, 0.f);
                if (use[k]) { // flags and the phase gather do not wait for the plan
                    const int2 sv = slot_v[t];
                    const int vx = (int)(short)(sv.x & 0xffff), vy = sv.x >> 16;
                    const int ux = w.x - vx, uy = w.y - vy;
                    const bool inu = !(ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1);
                    const int pu = inu ? wrap_idx(ux, uy, W, H) : 0, pv = sv.y;
                    use[k] = inu && flag(pu) && flag(pv);
                    ph[k] = use[k] ? phase(pu) : make_float2(0.f, 0.f);
                }
            }
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                if (!use[k] || (bh[k].x == 0.f && bh[k].y == 0.f)) // the plan's zero: never contributes
                    continue;
                if (isnan(bh[k].x)) {
                    record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                    continue;
                }
                const float2 p = cmul(cmul(ph[k], vtab[tt[k]]), make_float2(bh[k].x, -bh[k].y));
                const float r = rsqrtf(p.x * p.x + p.y * p.y);
                sr += p.x * r;
                si += p.y * r;
                ++cnt;
            }
        }
    };

    if (warp == 0) {
        // ------------------------------------------------ serial warp
        // Visit data that does not depend on the walk is loaded ahead: the
        // visit, its recent-pair count and slots two visits ahead, their plan
        // phasors one visit ahead.  Phases the walk just set come from a
        // shared-memory cache keyed by point (a miss reads the phase map).
        for (int i = lane; i < kPhaseCache; i += 32)
            pc_key[i] = -1;
        __syncwarp();
        struct Ahead {
            int2 w;
            int rc, ta, tb;
            float2 ba, bb;
        };
        // the list slots are loaded without waiting for the count (a visit's
        // kRecentMax entries are always allocated) and masked one visit later
        auto load_meta = [&](int q, Ahead& a) {
            if (q >= J.nvisits)
                return;
            a.w = J.visits[q];
            a.rc = J.rcount[q];
            const unsigned short* rl = J.rlist + (long long)q * kRecentMax;
            a.ta = rl[lane];
            a.tb = rl[lane + 32];
        };
        auto load_plan = [&](int q, Ahead& a) {
            if (q >= J.nvisits)
                return;
            a.ta = lane < a.rc ? a.ta : -1;
            a.tb = lane + 32 < a.rc ? a.tb : -1;
            const float2* prow = J.plan + (long long)q * nv;
            a.ba = a.ta >= 0 ? prow[a.ta] : make_float2(0.f, 0.f);
            a.bb = a.tb >= 0 ? prow[a.tb] : make_float2(0.f, 0.f);
        };
        Ahead c0 {}, c1 {}, c2 {};
        load_meta(0, c0);
        load_plan(0, c0);
        load_meta(1, c1);
        auto phase_of = [&](int p) {
            const int h = p & (kPhaseCache - 1);
            return pc_key[h] == p ? pc_val[h] : J.phf[p];
        };
        auto term_s = [&](int t, float2 bh, int2 w, float& sr, float& si, int& cnt) {
            if (bh.x == 0.f && bh.y == 0.f)
                return;
            const int2 sv = slot_v[t];
            const int vx = (int)(short)(sv.x & 0xffff), vy = sv.x >> 16;
            const int pu = wrap_idx(w.x - vx, w.y - vy, W, H), pv = sv.y;
            if (!flag(pu) || !flag(pv))
                return;
            if (isnan(bh.x)) {
                record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                return;
            }
            const float2 ph = cmul(cmul(phase_of(pu), vtab[t]), make_float2(bh.x, -bh.y));
            const float r = rsqrtf(ph.x * ph.x + ph.y * ph.y);
            sr += ph.x * r;
            si += ph.y * r;
            ++cnt;
        };
        for (int q = 0; q < J.nvisits; ++q) {
            load_plan(q + 1, c1); // its slots were loaded one visit ago
            load_meta(q + 2, c2);
            const int2 w = c0.w;
            bool run = !(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1);
            const int pw = run ? wrap_idx(w.x, w.y, W, H) : 0;
            run = run && !flag(pw);
            run = run && (abs(w.x) + abs(w.y) > 1);                                   // phasereco.h:84
            run = run && !(w.x < umn0 || w.x > umx0 || w.y < umn1 || w.y > umx1);
            if (run) {
                const int slot = q % kRing;
                if (!__all_sync(0xffffffffu, wait_until([&] { return ld_acquire_cta(&ring_tag[slot]) == q; }) ? 1 : 0))
                    break;
                float sr = 0.f, si = 0.f;
                int cnt = 0;
                if (c0.rc >= 0) {
                    if (c0.ta >= 0)
                        term_s(c0.ta, c0.ba, w, sr, si, cnt);
                    if (c0.tb >= 0)
                        term_s(c0.tb, c0.bb, w, sr, si, cnt);
                } else {
                    sum_pairs(q, w, false, phase_of, sr, si, cnt);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    sr += __shfl_xor_sync(0xffffffffu, sr, o);
                    si += __shfl_xor_sync(0xffffffffu, si, o);
                    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
                }
                if (lane == 0) {
                    // float-float: the non-recent share plus the recent one
                    const float4 o4 = ring_s[slot];
                    float rh = o4.x, rl = o4.y, ih = o4.z, il = o4.w;
                    ff_add(rh, rl, sr, 0.f);
                    ff_add(ih, il, si, 0.f);
                    cnt += ring_n[slot];
                    if (cnt > 0) {
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
                        pc_val[pw & (kPhaseCache - 1)] = pf;
                        pc_key[pw & (kPhaseCache - 1)] = pw;
                        flagbits[pw >> 5] |= 1u << (pw & 31);
                    }
                }
                __syncwarp();
            }
            // publish progress every 8 visits (a release store; the lag leaves
            // the slack)
            if (((q & 7) == 7 || q + 1 == J.nvisits) && lane == 0)
                st_release_cta(&progress, q + 1);
            __syncwarp();
            c0 = c1;
            c1 = c2;
        }
    } else {
        // ------------------------------------------- non-recent shares
        for (int q = warp - 1; q < J.nvisits; q += kRecoThreads / 32 - 1) {
            if (!__all_sync(0xffffffffu, wait_until([&] { return ld_acquire_cta(&progress) >= q - kRecoLag; }) ? 1 : 0))
                break;
            const int2 w = J.visits[q];
            const int rc = J.rcount[q];
            float sr = 0.f, si = 0.f;
            int cnt = 0;
            const bool inmap = !(w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1);
            if (rc >= 0 && inmap)
                sum_pairs(q, w, true, [&](int pu) { return J.phf[pu]; }, sr, si, cnt);
            // float-float over the lanes, lane 0's order
            float rh = sr, rl = 0.f, ih = si, il = 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float a = __shfl_xor_sync(0xffffffffu, rh, o), b = __shfl_xor_sync(0xffffffffu, rl, o);
                const float c = __shfl_xor_sync(0xffffffffu, ih, o), e = __shfl_xor_sync(0xffffffffu, il, o);
                ff_add(rh, rl, a, b);
                ff_add(ih, il, c, e);
                cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            }
            if (lane == 0) {
                const int slot = q % kRing;
                ring_s[slot] = make_float4(rh, rl, ih, il);
                ring_n[slot] = cnt;
                st_release_cta(&ring_tag[slot], q);
            }
            __syncwarp();
        }
    }
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

// ------------------------------------------ ring-parallel estimator (opt-in)
// A different estimator from the reference's spiral, offered as an option:
// the spiral's visits are grouped by the radius r at which NextRecoIndex makes
// them (one ring per r, each point once per ring), and every point of ring k
// is formed in parallel from the pairs whose u and v got their phases in
// rings before k.  The spiral also uses phases set earlier in the same ring,
// so the two differ; the phase difference is measured, not bounded by the
// reference.  fring[p]: the ring in which point p got its phase (seeds 0),
// -1 while it has none; only rings < k are read while ring k is written, so
// the result does not depend on the order in which the ring's warps run.
__global__ void ring_seed_kernel(const RecoJob* __restrict__ jobs, int* __restrict__ fring)
{
    const RecoJob J = jobs[0];
    if (threadIdx.x < 5) { // seeds (phasereco.h:42-54), as in the spiral walk
        const int sx[5] = { 0, 1, 0, -1, 0 }, sy[5] = { 0, 0, 1, 0, -1 };
        const int p = wrap_idx(sx[threadIdx.x], sy[threadIdx.x], J.W, J.H);
        const float im = threadIdx.x < 3 ? 0.f : -0.f;
        J.phf[p] = make_float2(1.f, im);
        J.sums[p] = make_float4(0.f, 0.f, 0.f, 0.f);
        J.cnt[p] = -1;
        fring[p] = 0;
    }
}

// One warp per visit of ring `ring`: rq[0..n) are the ring's visit indices.
__global__ void __launch_bounds__(256) ring_pass_kernel(const RecoJob* __restrict__ jobs, const int* __restrict__ rq,
                                                        int n, int ring, int* __restrict__ fring)
{
    const RecoJob J = jobs[0];
    const int gw = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (gw >= n) // whole warps leave together
        return;
    const int W = J.W, H = J.H, De = J.De, nside = De + 1, nv = nside * nside;
    const int q = rq[gw];
    const int2 w = J.visits[q];
    const int pmin0 = -(W >> 1), pmin1 = -(H >> 1);
    const int pmax0 = -W / 2 + W - 1, pmax1 = -H / 2 + H - 1;
    const int szW = (W / 2) * 2 + 1, szH = (H / 2) * 2 + 1;
    const int umn0 = -(szW / 2), umx0 = szW - szW / 2 - 1, umn1 = -(szH / 2), umx1 = szH - szH / 2 - 1;
    if (w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1)
        return;
    const int pw = wrap_idx(w.x, w.y, W, H);
    if (fring[pw] >= 0 || abs(w.x) + abs(w.y) <= 1                          // phasereco.h:84
        || w.x < umn0 || w.x > umx0 || w.y < umn1 || w.y > umx1)
        return;
    const float2* prow = J.plan + (long long)q * nv;
    float sr = 0.f, si = 0.f;
    int cnt = 0;
    // kB slots per lane at a time: every gather of the group is issued before
    // any is used, so their latencies overlap; the sums take the slots in
    // increasing order as a one-slot loop would
    constexpr int kB = 8;
    for (int t0 = lane; t0 < nv; t0 += 32 * kB) {
        float2 bh[kB], pa[kB], pb[kB];
        int fu[kB], fv[kB];
        bool use[kB];
#pragma unroll
        for (int k = 0; k < kB; ++k) {
            const int t = t0 + 32 * k;
            use[k] = t < nv;
            bh[k] = use[k] ? prow[t] : make_float2(0.f, 0.f);
            const int vx = -De / 2 + t % nside, vy = -De / 2 + t / nside;
            const int ux = w.x - vx, uy = w.y - vy;
            use[k] = use[k] && !(ux < pmin0 || ux > pmax0 || uy < pmin1 || uy > pmax1);
            const int pu = use[k] ? wrap_idx(ux, uy, W, H) : 0, pv = use[k] ? wrap_idx(vx, vy, W, H) : 0;
            fu[k] = use[k] ? fring[pu] : -1;
            fv[k] = use[k] ? fring[pv] : -1;
            pa[k] = use[k] ? J.phf[pu] : make_float2(0.f, 0.f);
            pb[k] = use[k] ? J.phf[pv] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < kB; ++k) {
            if (!use[k] || (bh[k].x == 0.f && bh[k].y == 0.f)) // the plan's zero: never contributes
                continue;
            if (fu[k] < 0 || fu[k] >= ring || fv[k] < 0 || fv[k] >= ring)
                continue;
            if (isnan(bh[k].x)) {
                record_error(J.err, SMIP_DEV_ERR_OUT_OF_RANGE);
                continue;
            }
            const float2 ph = cmul(cmul(pa[k], pb[k]), make_float2(bh[k].x, -bh[k].y));
            const float r = rsqrtf(ph.x * ph.x + ph.y * ph.y);
            sr += ph.x * r;
            si += ph.y * r;
            ++cnt;
        }
    }
    float rh = sr, rl = 0.f, ih = si, il = 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float a = __shfl_xor_sync(0xffffffffu, rh, o), b = __shfl_xor_sync(0xffffffffu, rl, o);
        const float c = __shfl_xor_sync(0xffffffffu, ih, o), e = __shfl_xor_sync(0xffffffffu, il, o);
        ff_add(rh, rl, a, b);
        ff_add(ih, il, c, e);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0 && cnt > 0) {
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
        fring[pw] = ring;
    }
}

// FP64 mean, consistency and phase of every point and the flag map, as the
// spiral walk's final pass forms them.
__global__ void ring_final_kernel(const RecoJob* __restrict__ jobs, const int* __restrict__ fring)
{
    const RecoJob J = jobs[0];
    const int np = J.W * J.H;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const unsigned char f = fring[p] >= 0 ? 1 : 0;
        J.flags[p] = f;
        if (!f)
            continue;
        const int n = J.cnt[p];
        if (n < 0) {
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

cudaError_t launch_ring_reco(const RecoJob* job_dev, int* fring, const int* rq, const std::vector<int>& roff, int W,
                             int H, cudaStream_t st)
{
    reco_plan_kernel<<<dim3(1024, 1), 256, 0, st>>>(job_dev);
    note_launches(1);
    cudaError_t e = cudaMemsetAsync(fring, 0xff, sizeof(int) * (size_t)W * H, st); // -1: no phase yet
    if (e != cudaSuccess)
        return e;
    ring_seed_kernel<<<1, 32, 0, st>>>(job_dev, fring);
    note_launches(1);
    for (size_t k = 1; k + 1 < roff.size(); ++k) {
        const int n = roff[k + 1] - roff[k];
        if (n <= 0)
            continue;
        ring_pass_kernel<<<(n * 32 + 255) / 256, 256, 0, st>>>(job_dev, rq + roff[k], n, (int)k, fring);
        note_launches(1);
    }
    const int np = W * H;
    ring_final_kernel<<<(np + 255) / 256 < 2048 ? (np + 255) / 256 : 2048, 256, 0, st>>>(job_dev, fring);
    note_launches(1);
    return cudaGetLastError();
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
    reco_recent_kernel<<<dim3(1024, njobs), 256, 0, st>>>(jobs_dev);
    note_launches(1);
    reco_rlist_kernel<<<dim3(256, njobs), 256, 0, st>>>(jobs_dev);
    note_launches(1);
    const size_t smem = (sizeof(float2) + sizeof(int2)) * nv + sizeof(unsigned int) * (((size_t)max_W * max_H + 31) / 32);
    // the limit is that of the largest frame and depth (the attribute is per
    // function; a launch of another shape must never lower it under this one);
    // the static shared memory (ring, phase cache) counts against it too
    const size_t smem_max = (sizeof(float2) + sizeof(int2)) * 65 * 65
                            + sizeof(unsigned int) * (((size_t)kMaxSide * kMaxSide + 31) / 32);
    if (max_De < kClusterDepth) { // one CTA per job
        cudaError_t e = cudaFuncSetAttribute(phase_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        if (e != cudaSuccess)
            return e;
        phase_pipe_kernel<<<njobs, kRecoThreads, smem, st>>>(jobs_dev);
        note_launches(1);
        return cudaGetLastError();
    }
    cudaError_t e = cudaFuncSetAttribute(phase_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    if (e != cudaSuccess)
        return e;
    // one cluster per job: kWalkCtas CTAs, or the largest power of two below
    // it that the GPU can place
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kRecoThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int ncta = kWalkCtas;
    for (; ncta > 1; ncta /= 2) {
        attr[0].val.clusterDim.x = ncta;
        cfg.gridDim = dim3(ncta);
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, phase_cluster_kernel, &cfg) == cudaSuccess && nclusters >= 1)
            break;
        cudaGetLastError();
    }
    attr[0].val.clusterDim.x = ncta;
    cfg.gridDim = dim3(njobs * ncta);
    e = cudaLaunchKernelEx(&cfg, phase_cluster_kernel, jobs_dev);
    note_launches(1);
    return e != cudaSuccess ? e : cudaGetLastError();
}

} // namespace smip_gpu
