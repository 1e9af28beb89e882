// k_bispec.cu -- bispectrum accumulation B(u,v) += F(u) F(v) conj F(u+v).
//
// Replaces Bispectrum<complex<float>>::accumulate_from_fft (include/
// bispectrum.h:356-409) for a batch of frames at once.
//
// Work decomposition.  The reference's loop runs over u = (i, j) with
// i in [-W/2, 0], j in [-H/2, H/2-1] and v = (k, l) with k in [-d/2, 0],
// l in [-d/2, d/2].  A tile is (a0 = -i, 16 consecutive j, a chunk of k rows);
// its bispectrum elements stay in registers while the frames of the batch
// stream through shared memory, so the packed bispectrum is read and written
// once per batch, not once per frame.
//
//   warp w            -> one k row (a2 = -k = chunk*KC + w)
//   lane (jg, lg)     -> j = j0 + jg + 4*tj (tj < 4),  l = -d/2 + lg + 8*tl (tl < d/8)
//   lanes 0..15       -> also the l = +d/2 column for j = j0 + lane
//
// With that mapping the 32 lanes of a warp read 11 consecutive F(u+v) words
// per shared-memory load (conflict-free), and each F(u+v) value held in a
// register serves up to four triple products.
//
// Per frame a dedicated producer warp issues three TMA box loads from the
// S[f][a][c] spectrum layout (k_fft.cu) into a ring of shared-memory stages:
//   W box: rows a0 + a2 (a2 in the chunk), columns j + l + H/2   -> F(u+v)
//   V box: rows a2,                        columns l + H/2       -> F(v)
//   A box: row a0,                         columns j + H/2       -> F(u)
// Out-of-range rows/columns are zero-filled by the TMA unit, which is exactly
// the reference's guard (bispectrum.h:397-398): those triples add zero.
//
// Accumulation: plain FP32 within a batch (in registers), Kahan-compensated
// across batches into (B, C) in HBM.  All mbarrier waits are bounded.
#include <cuda.h>

#include "smip_dev.cuh"

namespace smip_gpu {

constexpr uint64_t kWaitNs = 2000000000ull; // 2 s

template <int DE>
struct BCfg {
    static constexpr int KK = DE / 2 + 1;          // k rows
    static constexpr int NCH = (KK + 16) / 17;     // k chunks per (a0, j-tile)
    static constexpr int KC = (KK + NCH - 1) / NCH;
    static constexpr int J = 16;
    static constexpr int TL = DE / 8;
    static constexpr int NWV = 4 + 2 * (TL - 1);   // W values per thread per frame
    static constexpr int BW = J + DE + 2;
    static constexpr int BV = DE + 2;
    static constexpr int THREADS = (KC + 1) * 32;
    static constexpr int WBYTES = KC * BW * 8;
    static constexpr int VBYTES = KC * BV * 8;
    static constexpr int ABYTES = J * 8;
    static constexpr int WOFF = 0;
    static constexpr int VOFF = (WBYTES + 127) / 128 * 128;
    static constexpr int AOFF = VOFF + (VBYTES + 127) / 128 * 128;
    static constexpr int STAGE = AOFF + 128;
    // as many frame stages as ~200 KB of shared memory holds, 4..12
    static constexpr int NS = (200 * 1024 / STAGE) > 12 ? 12 : ((200 * 1024 / STAGE) < 4 ? 4 : (200 * 1024 / STAGE));
    static constexpr int SMEM = NS * STAGE + 2 * NS * 8;
};

struct BispecArgs {
    float2* B;
    float2* C;
    int* err;
    int nframes;
    int H, hw;
    int njt;      // H / 16
    int ntiles;
};

template <int DE>
__global__ void __launch_bounds__(BCfg<DE>::THREADS, 1)
    bispec_accum_kernel(const __grid_constant__ CUtensorMap tmW, const __grid_constant__ CUtensorMap tmV,
                        const __grid_constant__ CUtensorMap tmA, const BispecArgs p)
{
    using Cf = BCfg<DE>;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cf::NS * Cf::STAGE);
    uint64_t* empty = full + Cf::NS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < Cf::NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], Cf::KC);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int H = p.H;
    const int half_h = H / 2;

    if (warp == Cf::KC) { // ---------------------------------------- producer
        if (lane != 0)
            return;
        uint32_t it = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
            const int kc = t % Cf::NCH;
            const int rest = t / Cf::NCH;
            const int jt = rest % p.njt, a0 = rest / p.njt;
            const int j0 = -half_h + Cf::J * jt;
            const int cw = (j0 + half_h - DE / 2) & ~1;
            const int cv = (half_h - DE / 2) & ~1;
            for (int f = 0; f < p.nframes; ++f, ++it) {
                const int s = it % Cf::NS;
                const uint32_t use = it / Cf::NS;
                if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1) & 1, kWaitNs)) {
                    record_error(p.err, SMIP_DEV_ERR_TIMEOUT);
                    ok = false;
                    break;
                }
                unsigned char* st = smem + s * Cf::STAGE;
                mbar_arrive_expect_tx(&full[s], Cf::WBYTES + Cf::VBYTES + Cf::ABYTES);
                tma_load_3d(st + Cf::WOFF, &tmW, 2 * cw, a0 + kc * Cf::KC, f, &full[s]);
                tma_load_3d(st + Cf::VOFF, &tmV, 2 * cv, kc * Cf::KC, f, &full[s]);
                tma_load_3d(st + Cf::AOFF, &tmA, 2 * (j0 + half_h), a0, f, &full[s]);
            }
        }
        // let the last loads land before the block can retire
        const uint32_t first = it > (uint32_t)Cf::NS ? it - Cf::NS : 0;
        for (uint32_t q = first; q < it; ++q)
            mbar_wait_bounded(&full[q % Cf::NS], (q / Cf::NS) & 1, kWaitNs / 4);
        return;
    }

    // ------------------------------------------------------------ consumers
    const int jg = lane & 3, lg = lane >> 2;
    uint32_t it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const int kc = t % Cf::NCH;
        const int rest = t / Cf::NCH;
        const int jt = rest % p.njt, a0 = rest / p.njt;
        const int j0 = -half_h + Cf::J * jt;
        const int a2 = kc * Cf::KC + warp;
        const bool active = a2 < Cf::KK;
        const int offw = (j0 + half_h - DE / 2) - ((j0 + half_h - DE / 2) & ~1);
        const int offv = (half_h - DE / 2) - ((half_h - DE / 2) & ~1);

        float2 acc[4][Cf::TL];
        float2 acce = make_float2(0.f, 0.f);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < Cf::TL; ++b)
                acc[a][b] = make_float2(0.f, 0.f);

        for (int f = 0; f < p.nframes; ++f, ++it) {
            const int s = it % Cf::NS;
            const uint32_t use = it / Cf::NS;
            if (ok && !mbar_wait_bounded(&full[s], use & 1, kWaitNs)) {
                record_error(p.err, SMIP_DEV_ERR_TIMEOUT);
                ok = false;
            }
            if (!ok)
                break;
            const unsigned char* st = smem + s * Cf::STAGE;
            const float2* Wb = reinterpret_cast<const float2*>(st + Cf::WOFF) + warp * Cf::BW + offw;
            const float2* Vb = reinterpret_cast<const float2*>(st + Cf::VOFF) + warp * Cf::BV + offv;
            const float2* Ab = reinterpret_cast<const float2*>(st + Cf::AOFF);
            if (active) {
                float2 A[4], V[Cf::TL];
#pragma unroll
                for (int a = 0; a < 4; ++a)
                    A[a] = Ab[jg + 4 * a];
#pragma unroll
                for (int b = 0; b < Cf::TL; ++b)
                    V[b] = Vb[lg + 8 * b];
#pragma unroll
                for (int m = 0; m < Cf::NWV; ++m) {
                    const float2 w = Wb[jg + lg + 4 * m];
#pragma unroll
                    for (int b = 0; b < Cf::TL; ++b) {
                        const int a = m - 2 * b;
                        if (a >= 0 && a < 4) {
                            // t = F(u) F(v); acc += t * conj F(u+v)
                            const float tr = A[a].x * V[b].x - A[a].y * V[b].y;
                            const float ti = A[a].x * V[b].y + A[a].y * V[b].x;
                            acc[a][b].x = fmaf(tr, w.x, fmaf(ti, w.y, acc[a][b].x));
                            acc[a][b].y = fmaf(ti, w.x, fmaf(-tr, w.y, acc[a][b].y));
                        }
                    }
                }
                if (lane < 16) { // l = +d/2 column
                    const float2 ae = Ab[lane], ve = Vb[DE], we = Wb[DE + lane];
                    const float tr = ae.x * ve.x - ae.y * ve.y;
                    const float ti = ae.x * ve.y + ae.y * ve.x;
                    acce.x = fmaf(tr, we.x, fmaf(ti, we.y, acce.x));
                    acce.y = fmaf(ti, we.x, fmaf(-tr, we.y, acce.y));
                }
            }
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&empty[s]);
        }
        if (!ok)
            break;
        if (active) {
            // Kahan-compensated add of the batch partial into (B, C): every
            // load is issued before the first store (B and C never alias), so
            // the tile pays one memory round trip, not one per element.
            constexpr int rowE = (DE / 2 + 1) * (DE + 1);
            float2* __restrict__ Bt = p.B + ((long long)a0 * (H + 1)) * rowE + (long long)a2 * (DE + 1);
            float2* __restrict__ Ct = p.C + ((long long)a0 * (H + 1)) * rowE + (long long)a2 * (DE + 1);
            auto off = [&](int j, int l) {
                const int a1 = j >= 0 ? j : j + H + 1;
                const int a3 = l >= 0 ? l : l + DE + 1;
                return a1 * rowE + a3;
            };
            auto kahan = [](float2& b, float2& c, float2 v) {
                const float yx = v.x - c.x, yy = v.y - c.y;
                const float tx = b.x + yx, ty = b.y + yy;
                c.x = (tx - b.x) - yx;
                c.y = (ty - b.y) - yy;
                b = make_float2(tx, ty);
            };
            const int oe = off(j0 + (lane & 15), DE / 2);
            float2 be = make_float2(0.f, 0.f), ce = be;
            if (lane < 16) {
                be = Bt[oe];
                ce = Ct[oe];
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) { // two halves keep the register count down
                int o[2][Cf::TL];
                float2 bv[2][Cf::TL], cv[2][Cf::TL];
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < Cf::TL; ++b) {
                        o[a][b] = off(j0 + jg + 4 * (2 * h + a), -DE / 2 + lg + 8 * b);
                        bv[a][b] = Bt[o[a][b]];
                        cv[a][b] = Ct[o[a][b]];
                    }
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < Cf::TL; ++b) {
                        kahan(bv[a][b], cv[a][b], acc[2 * h + a][b]);
                        Bt[o[a][b]] = bv[a][b];
                        Ct[o[a][b]] = cv[a][b];
                    }
            }
            if (lane < 16) {
                kahan(be, ce, acce);
                Bt[oe] = be;
                Ct[oe] = ce;
            }
        }
    }
}

// ---------------------------------------------------------------- host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode()
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

// S viewed as FLOAT32 [nframes][hw][2H]; box = {2*bw floats, rows, 1 frame}
static bool make_map(CUtensorMap* m, const float2* S, int nframes, const Geometry& g, int bw, int rows)
{
    EncodeTiledFn enc = get_encode();
    if (!enc)
        return false;
    const cuuint64_t dims[3] = { (cuuint64_t)2 * g.H, (cuuint64_t)g.hw, (cuuint64_t)nframes };
    const cuuint64_t strides[2] = { (cuuint64_t)2 * g.H * 4, (cuuint64_t)2 * g.H * 4 * g.hw };
    const cuuint32_t box[3] = { (cuuint32_t)(2 * bw), (cuuint32_t)rows, 1 };
    const cuuint32_t es[3] = { 1, 1, 1 };
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float2*>(S), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE)
        == CUDA_SUCCESS;
}

template <int DE>
static cudaError_t launch_de(const BispecLaunch& L, const Geometry& g, cudaStream_t st)
{
    using Cf = BCfg<DE>;
    CUtensorMap mW, mV, mA;
    if (!make_map(&mW, L.S, L.nframes, g, Cf::BW, Cf::KC) || !make_map(&mV, L.S, L.nframes, g, Cf::BV, Cf::KC)
        || !make_map(&mA, L.S, L.nframes, g, Cf::J, 1))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(bispec_accum_kernel<DE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Cf::SMEM);
    if (e != cudaSuccess)
        return e;
    BispecArgs a;
    a.B = L.B;
    a.C = L.C;
    a.err = L.err;
    a.nframes = L.nframes;
    a.H = g.H;
    a.hw = g.hw;
    a.njt = g.H / Cf::J;
    a.ntiles = g.hw * a.njt * Cf::NCH;
    const int grid = a.ntiles < L.num_sms ? a.ntiles : L.num_sms;
    bispec_accum_kernel<DE><<<grid, Cf::THREADS, Cf::SMEM, st>>>(mW, mV, mA, a); note_launches(1);
    return cudaGetLastError();
}

bool bispec_depth_supported(int De) { return De >= 8 && De <= 64 && De % 8 == 0; }

cudaError_t launch_bispec_accumulate(const BispecLaunch& L, const Geometry& g, cudaStream_t st)
{
    if (L.nframes <= 0)
        return cudaSuccess;
    switch (g.De) {
    case 8: return launch_de<8>(L, g, st);
    case 16: return launch_de<16>(L, g, st);
    case 24: return launch_de<24>(L, g, st);
    case 32: return launch_de<32>(L, g, st);
    case 40: return launch_de<40>(L, g, st);
    case 48: return launch_de<48>(L, g, st);
    case 56: return launch_de<56>(L, g, st);
    case 64: return launch_de<64>(L, g, st);
    default: return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------- normalise, merge
__global__ void bispec_normalize_kernel(const float2* __restrict__ B, const float2* __restrict__ C, double n,
                                        long long count, float2* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const float2 b = B[i], c = C[i];
        out[i] = make_float2((float)(((double)b.x - (double)c.x) / n), (float)(((double)b.y - (double)c.y) / n));
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
    bispec_normalize_kernel<<<2048, 256, 0, st>>>(B, C, nframes, n, out); note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_bispec_merge(float2* Bd, float2* Cd, const float2* Bs, const float2* Cs, long long n,
                                cudaStream_t st)
{
    bispec_merge_kernel<<<2048, 256, 0, st>>>(Bd, Cd, Bs, Cs, n); note_launches(1);
    return cudaGetLastError();
}

} // namespace smip_gpu
