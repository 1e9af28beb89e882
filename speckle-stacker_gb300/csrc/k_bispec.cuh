// k_bispec.cuh -- bispectrum accumulation B(u,v) += F(u) F(v) conj F(u+v).
//
// Replaces Bispectrum<complex<float>>::accumulate_from_fft (include/
// bispectrum.h:356-409) for a batch of frames at once.
//
// The reference's loop runs over u = (i, j) with i in [-W/2, 0], j in
// [-H/2, H/2-1] and v = (k, l) with k in [-d/2, 0], l in [-d/2, d/2].
// Indices below: a0 = -i, a2 = -k.
//
// Work decomposition.  A warp task is (a0, a2, 32 consecutive j, one block of
// up to 32 l values); its triple sums stay in registers while the frames of
// the batch stream through shared memory, so the packed bispectrum is read and
// written once per batch, not once per frame.  A CTA has 16 warps (one CTA per
// SM: every SM sub-partition runs four equally loaded warps) and covers a tile
// of JT = 32 * NJB consecutive j:
//   main tile  (a0, j tile, chunk): rows a2 = 1..d/2 in chunks of RPC rows;
//   row-0 tile (a0 group, j tile):  row a2 = 0 for RPC consecutive a0.
// Warp w takes j block w % NJB and (l block, row) from w / NJB.  The grid has
// one CTA per tile, so the block scheduler places tiles on whichever SMs are
// free; the tiles of the last partial wave are split by frames into parts
// (one CTA each) whose partial sums are merged by the tile's last part.
//
//   lane (jg, lg) -> j = jw + jg + 4 a (a < 8),  l = -d/2 + 8 TLW lb + lg + 8 b (b < TLW)
//   every lane    -> also the l = +d/2 column for j = jw + lane (last l block)
//
// Each thread owns 32 triple sums (8 j x 4 l).  Per frame it loads 8 F(u),
// TLW F(v) and 8 + 2 (TLW - 1) F(u+v) values, 8 bytes each: the lanes of a warp
// read few distinct words per load (broadcasts), and every F(u+v) value in a
// register serves up to four triples.  Shared-memory traffic is about 6.5
// bytes per triple per lane, below the SM's 128 bytes per cycle at the FMA
// pipe's rate.  Plain FP32 (8 FMA-pipe instructions per triple).  A variant
// that formed F(u) F(v) with two packed fma.rn.f32x2 (its operand forms
// (vx, vx), (vy, vy), (-ay, ax) built once per frame, on the ALU pipe) cut
// the instructions by 9 % and the issue-active share from 74 % to 67 %, but
// its packed FMAs stalled on the math-pipe throttle (1.67 vs 0.04 warps per
// issue), the FMA pipe stayed 65 % active and the kernel ran 1 % slower
// (188.6k vs 190.5k frames/s at 256 x 256, depth 32), so the scalar form
// stays.
//
// Per ring stage, three TMA box loads from the S[f][a][c] spectrum layout
// (k_fft.cu; 8-byte elements) bring FPS = 4 frames (the box's outermost
// dimension), so the wait, the release and the stage's address arithmetic
// are paid once per four frames:
//   W box: rows a0 + a2, columns j + l + H/2   -> F(u+v)
//   V box: rows a2,      columns l + H/2       -> F(v)
//   A box: row a0,       columns j + H/2       -> F(u)  (row-0 tiles read F(u)
//          out of their W box, whose rows are the same a0 rows)
// Out-of-range rows/columns are zero-filled by the TMA unit, which is exactly
// the reference's guard (bispectrum.h:397-398): those triples add zero.  The
// ring is refilled round robin: the warp that finishes iteration r, r % 16 ==
// warp, issues iteration r + NS - LAG once every thread has released r - LAG.
//
// Accumulation: plain FP32 within a batch (in registers), Kahan-compensated
// across batches into (B, C) in HBM.  Every mbarrier wait is bounded.
#pragma once

#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "smip_dev.cuh"

namespace smip_gpu {

constexpr uint64_t kWaitNs = 2000000000ull; // 2 s

// Resident CTAs per SM, each with its own ring.  Two CTAs of 8 warps measured
// the same as one of 16 (189.5k vs 189.7k frames/s at 256x256, d = 32).
constexpr int kCtasPerSm = 1;

// FPSV: frames per ring stage (4 by default; the autotuner may pick 2).  The
// tile geometry does not depend on it, and neither do results: a thread adds
// its frames in frame order whatever the staging.
template <int DE, int FPSV = 4>
struct BCfg {
    static constexpr int ROWS = DE / 2;                    // main rows a2 = 1..d/2
    static constexpr int TL = DE / 8;                      // 8-wide l groups in [-d/2, d/2)
    static constexpr int NLB = (TL + 3) / 4;               // l blocks per row
    static constexpr int TLW = (TL + NLB - 1) / NLB;       // l groups per block
    static constexpr int RPC = (NLB == 1 && ROWS % 8 == 0) ? 8 : 4; // rows (a0 for row-0 tiles) per tile
    static constexpr int WARPS = 16 / kCtasPerSm;
    static constexpr int NJB = WARPS / (RPC * NLB);        // 32-wide j blocks per tile
    static constexpr int JT = 32 * NJB;                    // tile j width
    static constexpr int THREADS = WARPS * 32;
    static constexpr int NWV = 8 + 2 * (TLW - 1);          // W values per thread per frame
    static constexpr int BW = JT + DE + 2;                 // W box columns (even start)
    static constexpr int BV = DE + 2;                      // V box columns (even start)
    static constexpr int FPS = FPSV;                       // frames per ring stage
    static constexpr int WBYTES = RPC * BW * 8;            // one frame's boxes
    static constexpr int VBYTES = RPC * BV * 8;
    static constexpr int ABYTES = JT * 8;
    static constexpr int WOFF = 0;
    static constexpr int VOFF = (FPS * WBYTES + 127) / 128 * 128;
    static constexpr int AOFF = VOFF + (FPS * VBYTES + 127) / 128 * 128;
    static constexpr int STAGE = AOFF + (FPS * ABYTES + 127) / 128 * 128;
    static constexpr int NSR = (200 * 1024 / kCtasPerSm) / STAGE; // ~200 KB of frame stages per SM
    static constexpr int NS = NSR > 16 ? 16 : (NSR < 4 ? 4 : NSR);
    static constexpr int LAG = 2;                          // iterations between a stage's release and its refill
                                                           // (3 at d = 32, with 6 stages, measured no faster)
    static constexpr int SMEM = NS * STAGE + 2 * NS * 8 + 16;
    static_assert(RPC * NLB * NJB == WARPS && ROWS % RPC == 0, "task split");
    static_assert(BW <= 256 && NS > LAG + 1 && SMEM <= (227 * 1024) / kCtasPerSm - 1024, "box / ring");
};

struct BispecArgs {
    float2* B;
    float2* C;
    int* err;
    int nframes;
    int H, hw;
    int bs1;      // packed extent of u_y: (H/2)*2 + 1
    int D;        // the stack's depth (even, <= DE): packed layout and stored elements
    int nchm;     // main chunks per (a0, j tile): ceil((D/2) / RPC)
    int njt;      // j tiles: ceil(H / JT)
    // Main tiles list only chunks whose first row has u + v inside the
    // spectrum (a0 + a2 <= hw - 1); the others would add nothing but zeros.
    // a0 < areg: all nchm chunks (nreg tiles); a0 in [areg, hw - 2]: fewer.
    int areg, nreg;
    int nmain;    // main tiles
    int ntiles;   // main + row-0 tiles
    // Work units, one CTA each: tiles [0, nfull) whole; the remaining tiles
    // (a last partial wave of the GPU) split by frames into P parts each
    // (nsplit units).  Parts write partial sums to scratch; the CTA that
    // completes a tile's last part adds the parts, in part order, into (B, C).
    int nfull, P, nsplit;
    float2* scratch;   // [nsplit][NSLOT][THREADS] partial sums
    int* tile_cnt;     // [ntiles - nfull] parts finished (zero between launches)
};

// Tile geometry shared by the TMA issue path and the consumers.
struct TileInfo {
    bool row0;
    int a0;   // main: the tile's a0; row-0: first a0 of the group
    int j0;
    int c;    // main: chunk
};

// Chunks c of a0 whose first row a2 = 1 + c RPC keeps a0 + a2 <= hw - 1.
template <int DE>
__host__ __device__ inline int main_chunks(int a0, int hw, int nchm)
{
    if (a0 > hw - 2)
        return 0;
    const int nc = (hw - 2 - a0) / BCfg<DE>::RPC + 1;
    return nc < nchm ? nc : nchm;
}

template <int DE>
__device__ __forceinline__ TileInfo decode_tile(int t, const BispecArgs& p)
{
    using Cf = BCfg<DE>;
    TileInfo ti;
    ti.row0 = t >= p.nmain;
    int jt;
    if (!ti.row0 && t < p.nreg) {
        ti.c = t % p.nchm;
        const int rest = t / p.nchm;
        jt = rest % p.njt;
        ti.a0 = rest / p.njt;
    } else if (!ti.row0) { // the last a0 rows: chunks [0, main_chunks(a0)) each
        int u = t - p.nreg, a0 = p.areg;
        for (;;) {
            const int nc = main_chunks<DE>(a0, p.hw, p.nchm);
            if (u < nc * p.njt) {
                jt = u / nc;
                ti.c = u % nc;
                break;
            }
            u -= nc * p.njt;
            ++a0;
        }
        ti.a0 = a0;
    } else {
        const int t0 = t - p.nmain;
        ti.c = 0;
        jt = t0 % p.njt;
        ti.a0 = (t0 / p.njt) * Cf::RPC;
    }
    ti.j0 = -(p.H / 2) + Cf::JT * jt;
    return ti;
}

__device__ __forceinline__ void cmac(float2& acc, float2 a, float2 v, float2 w)
{
    // t = a v;  acc += t conj(w)
    const float tr = a.x * v.x - a.y * v.y;
    const float ti = a.x * v.y + a.y * v.x;
    acc.x = fmaf(tr, w.x, fmaf(ti, w.y, acc.x));
    acc.y = fmaf(ti, w.x, fmaf(-tr, w.y, acc.y));
}

// One unit of work -- tile `unit` whole, or a frame part of a split tile --
// by all threads of the block: ring set-up, the frame loop and the
// Kahan-compensated epilogue.  EXACT: the stack's depth is DE itself
// (compile-time layout); otherwise the depth comes from the arguments
// (BispecArgs::D < DE).  Returns false when a bounded wait expired (the
// error is recorded in p.err).  On return every copy this unit issued has
// landed and the ring's barriers are invalidated, so the shared memory can
// take the next unit.
template <int DE, bool EXACT, int FPSV = 4>
__device__ __forceinline__ bool bispec_unit(unsigned char* smem, const CUtensorMap* tmW, const CUtensorMap* tmV,
                                            const CUtensorMap* tmA, const BispecArgs& p, const int unit)
{
    using Cf = BCfg<DE, FPSV>;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cf::NS * Cf::STAGE);
    uint64_t* empty = full + Cf::NS;
    uint32_t* hi_issued = reinterpret_cast<uint32_t*>(empty + Cf::NS); // highest iteration issued + 1
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < Cf::NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], Cf::THREADS); // every consumer thread releases its own reads
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int half_h = p.H / 2;
    const int jend = p.H - half_h; // u_y in [-(H/2), jend)
    const int nf = p.nframes;
    // this CTA's unit: tile unit whole, or (split unit s = unit -
    // nfull) part s % P of tile nfull + s / P, frames [part*nf/P, (part+1)*nf/P)
    const bool split_unit = (int)unit >= p.nfull;
    auto split_s = [&]() { return (int)unit - p.nfull; };
    auto split_tile = [&]() { return p.nfull + split_s() / p.P; };
    auto split_f0 = [&]() { return (int)((long long)(split_s() % p.P) * nf / p.P); };
    auto split_f1 = [&]() { return (int)((long long)(split_s() % p.P + 1) * nf / p.P); };
    const uint32_t total = split_unit ? (uint32_t)(split_f1() - split_f0()) : (uint32_t)nf;
    const uint32_t niter = (total + Cf::FPS - 1) / Cf::FPS; // ring iterations (FPS frames each)
    const int cv = (half_h - DE / 2) & ~1;
    const int offv = (half_h - DE / 2) - cv;

    // box coordinates of this CTA's tile, set once by thread 0 (x in 8-byte
    // elements, even: 16-byte aligned); iteration r loads frames f0 + FPS r ..
    // f0 + FPS r + FPS - 1 (one box per operand, frames outermost)
    __shared__ int s_box[7]; // W x, W y, V y, A x, A y, f0, row-0 tile

    // issue the loads of iteration r into stage r % NS
    auto issue = [&](uint32_t r) {
        const int f = s_box[5] + Cf::FPS * (int)r;
        const int s = r % Cf::NS;
        unsigned char* st = smem + s * Cf::STAGE;
        if (!s_box[6]) {
            mbar_arrive_expect_tx(&full[s], Cf::FPS * (Cf::WBYTES + Cf::VBYTES + Cf::ABYTES));
            tma_load_3d(st + Cf::WOFF, tmW, s_box[0], s_box[1], f, &full[s]);
            tma_load_3d(st + Cf::VOFF, tmV, cv, s_box[2], f, &full[s]);
            tma_load_3d(st + Cf::AOFF, tmA, s_box[3], s_box[4], f, &full[s]);
        } else {
            mbar_arrive_expect_tx(&full[s], Cf::FPS * (Cf::WBYTES + Cf::VBYTES));
            tma_load_3d(st + Cf::WOFF, tmW, s_box[0], s_box[1], f, &full[s]);
            tma_load_3d(st + Cf::VOFF, tmV, cv, s_box[2], f, &full[s]);
        }
    };

    // The first NS - LAG iterations are issued up front; afterwards the warp
    // that finishes iteration r with r % WARPS == warp issues r + NS - LAG.
    constexpr uint32_t kAhead = Cf::NS - Cf::LAG;
    if (threadIdx.x == 0) {
        const TileInfo ti = decode_tile<DE>(split_unit ? split_tile() : (int)unit, p);
        s_box[0] = (ti.j0 + half_h - DE / 2) & ~1;
        s_box[1] = ti.row0 ? ti.a0 : ti.a0 + 1 + ti.c * Cf::RPC;
        s_box[2] = ti.row0 ? 0 : 1 + ti.c * Cf::RPC;
        s_box[3] = ti.j0 + half_h;
        s_box[4] = ti.a0;
        s_box[5] = split_unit ? split_f0() : 0;
        s_box[6] = ti.row0;
        const uint32_t n0 = niter < kAhead ? niter : kAhead;
        for (uint32_t q = 0; q < n0; ++q)
            issue(q);
        *hi_issued = n0;
    }
    uint32_t nr = (uint32_t)warp + kAhead; // this warp's next refill
    bool stop = false;
    __syncthreads();

    const int jg = lane & 3, lg = lane >> 2;
    const int jb = warp % Cf::NJB;
    const int lb = (warp / Cf::NJB) % Cf::NLB;
    const int wr = warp / (Cf::NJB * Cf::NLB); // row inside the tile's boxes
    const int nb = Cf::TLW < Cf::TL - Cf::TLW * lb ? Cf::TLW : Cf::TL - Cf::TLW * lb; // valid l groups
    const bool edge = lb == Cf::NLB - 1;
    uint32_t r = 0;
    bool ok = true;
    __shared__ int s_last; // this CTA completes its split tile
    for (int k = 0; k < 1 && ok; ++k) {
        const int nfu = (int)total; // frames of this unit
        const TileInfo ti = decode_tile<DE>(split_unit ? split_tile() : (int)unit, p);
        const int a0 = ti.row0 ? ti.a0 + wr : ti.a0;
        const int a2 = ti.row0 ? 0 : 1 + ti.c * Cf::RPC + wr;
        const int vrow = ti.row0 ? 0 : wr;
        const int jw = ti.j0 + 32 * jb; // first j of this warp
        const int cw = (ti.j0 + half_h - DE / 2) & ~1;
        const int offw = (ti.j0 + half_h - DE / 2) - cw;
        // element offsets inside a stage (8-byte units)
        const int wbase = wr * Cf::BW + offw + 32 * jb;                 // W at (j = jw, l = -d/2)
        const int vbase = Cf::VOFF / 8 + vrow * Cf::BV + offv;         // V at l = -d/2
        const int abase = ti.row0 ? wbase + DE / 2 : Cf::AOFF / 8 + 32 * jb; // A at j = jw
        const int D = EXACT ? DE : p.D;
        const int hd = D / 2; // a depth below DE computes the template's extra rows and columns, stores none
        // A warp whose row has u + v outside the spectrum (every F(u+v) zero),
        // or whose row or j block lies outside the stack's layout, only keeps
        // the ring moving: its sums would be zero or unused.
        const bool live = a0 < p.hw && jw < jend && a0 + a2 < p.hw && (EXACT || a2 <= hd);

        float2 acc[8][Cf::TLW];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < Cf::TLW; ++b)
                acc[a][b] = make_float2(0.f, 0.f);
        float2 acce = make_float2(0.f, 0.f);

        // one frame of the stage: boxes at W, V, A (the row-0 tiles' A is in the W box)
        auto frame = [&](const float2* Wf, const float2* Vf, const float2* Af) {
            const float2* Wb = Wf + wbase + 8 * Cf::TLW * lb;
            const float2* Vb = Vf + vbase + 8 * Cf::TLW * lb;
            const float2* Ab = Af + abase;
            float2 A[8], V[Cf::TLW];
#pragma unroll
            for (int a = 0; a < 8; ++a)
                A[a] = Ab[jg + 4 * a];
#pragma unroll
            for (int b = 0; b < Cf::TLW; ++b)
                V[b] = b < nb ? Vb[lg + 8 * b] : make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m < Cf::NWV; ++m) {
                const float2 w = Wb[jg + lg + 4 * m];
#pragma unroll
                for (int b = 0; b < Cf::TLW; ++b) {
                    const int a = m - 2 * b;
                    if (a >= 0 && a < 8 && b < nb)
                        cmac(acc[a][b], A[a], V[b], w);
                }
            }
            if (edge) // l = +d/2 column, j = jw + lane
                cmac(acce, Af[abase + lane], Vf[vbase + DE], Wf[wbase + DE + lane]);
        };
        // the A box step between frames: in the W box for row-0 tiles
        const int astep = ti.row0 ? Cf::WBYTES / 8 : Cf::ABYTES / 8;

        for (uint32_t q = 0; q < niter; ++q, ++r) {
            const int s = r % Cf::NS;
            // every lane waits; the warp leaves together if any lane timed out
            const bool got = mbar_wait_bounded(&full[s], (r / Cf::NS) & 1, kWaitNs);
            if (!__all_sync(0xffffffffu, got)) {
                if (lane == 0)
                    record_error(p.err, SMIP_DEV_ERR_TIMEOUT);
                ok = false;
                break;
            }
            if (live) {
                const float2* st = reinterpret_cast<const float2*>(smem + s * Cf::STAGE);
                frame(st, st, st);
#pragma unroll
                for (int k = 1; k < Cf::FPS; ++k) // a unit's last stage may hold frames that are not its own
                    if (Cf::FPS * q + k < (uint32_t)nfu)
                        frame(st + k * (Cf::WBYTES / 8), st + k * (Cf::VBYTES / 8), st + k * astep);
            }
            // Each thread releases the stage itself: its arrive (release
            // semantics) orders its own shared-memory reads before the refill.
            // A single arrive per warp after __syncwarp measured unsafe: the
            // stage was overwritten under the reads of other lanes.
            mbar_arrive(&empty[s]);
            __syncwarp();
            if (r + kAhead == nr) { // ring refill, round robin over the warps
                if (!stop && nr < niter) {
                    bool go = true;
                    if (lane == 0) {
                        const uint32_t prev = r - Cf::LAG; // the iteration that last used the stage
                        if (r >= (uint32_t)Cf::LAG
                            && !mbar_wait_bounded(&empty[prev % Cf::NS], (prev / Cf::NS) & 1, kWaitNs)) {
                            record_error(p.err, SMIP_DEV_ERR_TIMEOUT);
                            go = false;
                        } else {
                            // generic-proxy reads of the stage before the async-proxy (TMA) writes
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            issue(nr);
                            atomicMax(hi_issued, nr + 1);
                        }
                    }
                    stop = !__shfl_sync(0xffffffffu, go, 0);
                }
                nr += Cf::WARPS;
            }
        }
        if (!ok)
            break;
        if (split_unit && p.P > 1) {
            // write this part's sums; the CTA that finishes the tile's last part merges
            constexpr int NSLOT = 8 * Cf::TLW + 1;
            const int b = split_s(), s_part = b % p.P, s_tile = split_tile();
            float2* sc = p.scratch + (long long)b * NSLOT * Cf::THREADS + threadIdx.x;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int q = 0; q < Cf::TLW; ++q)
                    sc[(a * Cf::TLW + q) * Cf::THREADS] = acc[a][q];
            sc[(NSLOT - 1) * Cf::THREADS] = acce;
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0)
                s_last = atomicAdd(&p.tile_cnt[s_tile - p.nfull], 1) == p.P - 1;
            __syncthreads();
            if (!s_last)
                continue;
            __threadfence();
            // parts in order 0..P-1: a fixed summation order whichever CTA merges
            const float2* sb = p.scratch + (long long)(b - s_part) * NSLOT * Cf::THREADS + threadIdx.x;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int q = 0; q < Cf::TLW; ++q)
                    acc[a][q] = make_float2(0.f, 0.f);
            acce = make_float2(0.f, 0.f);
            for (int pp = 0; pp < p.P; ++pp) {
                const float2* sp = sb + (long long)pp * NSLOT * Cf::THREADS;
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int q = 0; q < Cf::TLW; ++q) {
                        const float2 v = __ldcg(sp + (a * Cf::TLW + q) * Cf::THREADS);
                        acc[a][q].x += v.x;
                        acc[a][q].y += v.y;
                    }
                const float2 v = __ldcg(sp + (NSLOT - 1) * Cf::THREADS);
                acce.x += v.x;
                acce.y += v.y;
            }
            if (threadIdx.x == 0)
                p.tile_cnt[s_tile - p.nfull] = 0; // ready for the next launch
        }
        if (live) {
            // Kahan-compensated add of the batch partial into (B, C); within a
            // j step every load is issued before the first store (B and C never
            // alias).
            const int rowE = (hd + 1) * (D + 1);
            float2* __restrict__ Bt = p.B + ((long long)a0 * p.bs1) * rowE + (long long)a2 * (D + 1);
            float2* __restrict__ Ct = p.C + ((long long)a0 * p.bs1) * rowE + (long long)a2 * (D + 1);
            auto off = [&](int j, int l) {
                const int a1 = j >= 0 ? j : j + p.bs1;
                const int a3 = l >= 0 ? l : l + D + 1;
                return a1 * rowE + a3;
            };
            auto kahan = [](float2& b, float2& c, float2 v) {
                const float yx = v.x - c.x, yy = v.y - c.y;
                const float tx = b.x + yx, ty = b.y + yy;
                c.x = (tx - b.x) - yx;
                c.y = (ty - b.y) - yy;
                b = make_float2(tx, ty);
            };
            // a tile may reach past the last u_y when H < JT: those sums are zero and not stored
            const bool has_e = edge && jw + lane < jend && DE == D;
            const int oe = off(jw + lane, DE / 2);
            float2 be = make_float2(0.f, 0.f), ce = be;
            if (has_e) {
                be = Bt[oe];
                ce = Ct[oe];
            }
#pragma unroll
            for (int a = 0; a < 8; ++a) { // one j at a time keeps the register count down
                const int j = jw + jg + 4 * a;
                if (j < jend) {
                    int o[Cf::TLW];
                    float2 bv[Cf::TLW], cvv[Cf::TLW];
                    bool st[Cf::TLW];
#pragma unroll
                    for (int b = 0; b < Cf::TLW; ++b) {
                        const int l = -DE / 2 + 8 * Cf::TLW * lb + lg + 8 * b;
                        st[b] = b < nb && (EXACT || (l >= -hd && l <= hd));
                        if (st[b]) {
                            o[b] = off(j, l);
                            bv[b] = Bt[o[b]];
                            cvv[b] = Ct[o[b]];
                        }
                    }
#pragma unroll
                    for (int b = 0; b < Cf::TLW; ++b)
                        if (st[b]) {
                            kahan(bv[b], cvv[b], acc[a][b]);
                            Bt[o[b]] = bv[b];
                            Ct[o[b]] = cvv[b];
                        }
                }
            }
            if (has_e) {
                kahan(be, ce, acce);
                Bt[oe] = be;
                Ct[oe] = ce;
            }
        }
    }
    // On an early exit (a timed-out wait), loads may still be in flight: only
    // the last NS issued iterations can be, so wait (bounded) for those to land
    // before the block retires.
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t hi = *hi_issued;
        for (uint32_t q = hi > (uint32_t)Cf::NS ? hi - Cf::NS : 0; q < hi; ++q)
            if (!mbar_wait_bounded(&full[q % Cf::NS], (q / Cf::NS) & 1, kWaitNs / 4))
                break;
        for (int q = 0; q < 2 * Cf::NS; ++q) // the next unit initialises them afresh
            mbar_inval(&full[q]);
    }
    __syncthreads();
    return ok;
}

template <int DE, bool EXACT, int FPSV>
__global__ void __launch_bounds__(BCfg<DE, FPSV>::THREADS, kCtasPerSm)
    bispec_accum_kernel(const __grid_constant__ CUtensorMap tmW, const __grid_constant__ CUtensorMap tmV,
                        const __grid_constant__ CUtensorMap tmA, const BispecArgs p)
{
    extern __shared__ __align__(128) unsigned char smem[];
    bispec_unit<DE, EXACT, FPSV>(smem, &tmW, &tmV, &tmA, p, (int)blockIdx.x);
}

// ---------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static inline EncodeTiledFn get_encode()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess
            && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// S viewed as UINT64 (one complex<float> per element) [nframes][hw][Hs], H
// columns used (Hs = H rounded up to even keeps the strides multiples of 16
// bytes); box = {bcols, brows, nfb frames}.
static inline bool make_map(CUtensorMap* m, const float2* S, int nframes, const Geometry& g, int bcols, int brows, int nfb)
{
    EncodeTiledFn enc = get_encode();
    if (!enc)
        return false;
    const cuuint64_t dims[3] = { (cuuint64_t)g.H, (cuuint64_t)g.hw, (cuuint64_t)nframes };
    const cuuint64_t strides[2] = { (cuuint64_t)g.Hs * 8, (cuuint64_t)g.Hs * 8 * g.hw };
    const cuuint32_t box[3] = { (cuuint32_t)bcols, (cuuint32_t)brows, (cuuint32_t)nfb };
    const cuuint32_t es[3] = { 1, 1, 1 };
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<float2*>(S), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE)
        == CUDA_SUCCESS;
}

// The launch arguments of one batch: packed layout, tile list and the split
// of the last partial wave's tiles by frames.
template <int DE>
static inline BispecArgs fill_args(const BispecLaunch& L, const Geometry& g)
{
    using Cf = BCfg<DE>;
    BispecArgs a;
    a.B = L.B;
    a.C = L.C;
    a.err = L.err;
    a.nframes = L.nframes;
    a.H = g.H;
    a.hw = g.hw;
    a.bs1 = g.bs1;
    a.D = g.De;
    a.nchm = (g.De / 2 + Cf::RPC - 1) / Cf::RPC;
    a.njt = (g.H + Cf::JT - 1) / Cf::JT;
    a.areg = std::max(0, g.hw - 1 - (a.nchm - 1) * Cf::RPC);
    a.nreg = a.areg * a.njt * a.nchm;
    a.nmain = a.nreg;
    for (int a0 = a.areg; a0 < g.hw; ++a0)
        a.nmain += main_chunks<DE>(a0, g.hw, a.nchm) * a.njt;
    a.ntiles = a.nmain + (g.hw + Cf::RPC - 1) / Cf::RPC * a.njt;
    // One CTA per unit (not persistent, so the block scheduler can place tiles
    // on whichever SMs are free, also while other streams' kernels run).  The
    // tiles of the last partial wave (one CTA per SM) are split by frames so
    // that the wave is full (parts of at least 8 frames).
    const int G = L.num_sms * kCtasPerSm; // CTAs of one full wave
    const int rem = a.ntiles % G;
    int P = rem > 0 ? G / rem : 1;
    P = P < 1 ? 1 : P;
    const int minp = L.min_part > 0 ? L.min_part : 8; // frames per part at least
    const int pmax = L.nframes / minp > 1 ? L.nframes / minp : 1;
    P = P > pmax ? pmax : P;
    if (!L.scratch || !L.tile_cnt)
        P = 1;
    a.nfull = a.ntiles - (P > 1 ? rem : 0);
    a.P = P;
    a.nsplit = P > 1 ? rem * P : 0;
    a.scratch = L.scratch;
    a.tile_cnt = L.tile_cnt;
    return a;
}

template <int DE, int FPSV = 4>
static inline bool make_maps(CUtensorMap* m, const BispecLaunch& L, const Geometry& g)
{
    using Cf = BCfg<DE, FPSV>;
    return make_map(&m[0], L.S, L.nframes, g, Cf::BW, Cf::RPC, Cf::FPS)
           && make_map(&m[1], L.S, L.nframes, g, Cf::BV, Cf::RPC, Cf::FPS)
           && make_map(&m[2], L.S, L.nframes, g, Cf::JT, 1, Cf::FPS);
}

template <int DE, bool EXACT, int FPSV>
static cudaError_t launch_de(const BispecLaunch& L, const Geometry& g, cudaStream_t st)
{
    using Cf = BCfg<DE, FPSV>;
    CUtensorMap m[3];
    if (!make_maps<DE, FPSV>(m, L, g))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(bispec_accum_kernel<DE, EXACT, FPSV>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, Cf::SMEM);
    if (e != cudaSuccess)
        return e;
    const BispecArgs a = fill_args<DE>(L, g);
    const int grid = a.nfull + a.nsplit;
    bispec_accum_kernel<DE, EXACT, FPSV><<<grid, Cf::THREADS, Cf::SMEM, st>>>(m[0], m[1], m[2], a); note_launches(1);
    return cudaGetLastError();
}

// Every depth class for one staging variant: the kernel is instantiated for
// depths that are multiples of 8; another even depth runs the next one up and
// stores only its own elements.
template <int FPSV>
static cudaError_t launch_variant(const BispecLaunch& L, const Geometry& g, cudaStream_t st)
{
    const bool exact = g.De % 8 == 0;
    switch ((g.De + 7) / 8 * 8) {
    case 8: return exact ? launch_de<8, true, FPSV>(L, g, st) : launch_de<8, false, FPSV>(L, g, st);
    case 16: return exact ? launch_de<16, true, FPSV>(L, g, st) : launch_de<16, false, FPSV>(L, g, st);
    case 24: return exact ? launch_de<24, true, FPSV>(L, g, st) : launch_de<24, false, FPSV>(L, g, st);
    case 32: return exact ? launch_de<32, true, FPSV>(L, g, st) : launch_de<32, false, FPSV>(L, g, st);
    case 40: return exact ? launch_de<40, true, FPSV>(L, g, st) : launch_de<40, false, FPSV>(L, g, st);
    case 48: return exact ? launch_de<48, true, FPSV>(L, g, st) : launch_de<48, false, FPSV>(L, g, st);
    case 56: return exact ? launch_de<56, true, FPSV>(L, g, st) : launch_de<56, false, FPSV>(L, g, st);
    case 64: return exact ? launch_de<64, true, FPSV>(L, g, st) : launch_de<64, false, FPSV>(L, g, st);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace smip_gpu
