// smip_dev.cuh -- device helpers shared by the SMIP kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "smip_internal.h"

namespace smip_gpu {

// ---------------------------------------------------------------- complex ops
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <typename C> struct real_of;
template <> struct real_of<float2> { using type = float; };
template <> struct real_of<double2> { using type = double; };

__device__ __forceinline__ unsigned bitrev(unsigned i, int logn) { return __brev(i) >> (32 - logn); }

// In-place radix-2 decimation-in-time FFT of nl lines of length n = 1<<logn
// held in shared memory (line stride ls), input already in bit-reversed order.
// tw[k] = exp(-2*pi*i*k / 2^twlog) for k < 2^(twlog-1); sign -1 forward, +1
// inverse (unnormalised).  Called by all threads of the block.
template <typename C>
__device__ void fft_stages(C* buf, int logn, int nl, int ls, const C* tw, int twlog, int sign)
{
    const int n = 1 << logn;
    const int nb = nl * (n >> 1);
    for (int s = 1; s <= logn; ++s) {
        const int half = 1 << (s - 1);
        const int tsh = twlog - s;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            const int line = b >> (logn - 1);
            const int q = b & ((n >> 1) - 1);
            const int k = q & (half - 1);
            const int i0 = ((q >> (s - 1)) << s) + k;
            C w = tw[k << tsh];
            if (sign > 0)
                w.y = -w.y;
            C* L = buf + line * ls;
            const C a = L[i0];
            const C t = cmul(L[i0 + half], w);
            L[i0] = cadd(a, t);
            L[i0 + half] = csub(a, t);
        }
        __syncthreads();
    }
}

// ------------------------------------------------ float-float (~44-bit) FFT
// A value is hi + lo with |lo| <= ulp(hi)/2.  two_sum / two_prod are the
// error-free transformations of Knuth and Dekker (two_prod via FMA); products
// drop only the lo*lo term.  Used for the forward frame FFT so that weak
// frequency bins keep full FP32 relative accuracy after rounding, as an FP64
// transform narrowed to FP32 would give them.
// The error-free steps use __fadd_rn / __fsub_rn / __fmul_rn, which the
// compiler never contracts into an FMA with a neighbouring product (a
// contracted p + e would silently drop the low word).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& rh, float& rl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    rh = __fadd_rn(s, e);
    rl = __fsub_rn(e, __fsub_rn(rh, s));
}

__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& rh, float& rl)
{
    const float p = __fmul_rn(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, fmaf(al, bh, e));
    rh = __fadd_rn(p, e);
    rl = __fsub_rn(e, __fsub_rn(rh, p));
}

// The FFT butterflies below keep their values as unevaluated pairs hi + lo
// and skip the renormalisation (hi, lo) -> (fl(hi + lo), rest) after each
// operation: every hi + hi is still an error-free two_sum and every product
// an FMA-exact two_prod, and the lo words (a few ulps of hi) only collect
// those errors and the cross terms, so the pair keeps ~44-bit accuracy at
// 64 instead of 94 FP32 operations per butterfly.  Consumers round hi + lo
// once (df_round) or renormalise with df_norm before a product of pairs.
__device__ __forceinline__ void df_norm(float& h, float& l)
{
    float s, e;
    two_sum(h, l, s, e);
    h = s;
    l = e;
}

__device__ __forceinline__ void df_add_lazy(float ah, float al, float bh, float bl, float& rh, float& rl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    rh = s;
    rl = __fadd_rn(e, __fadd_rn(al, bl));
}

__device__ __forceinline__ dfc df_cadd(const dfc& a, const dfc& b)
{
    dfc r;
    df_add_lazy(a.h.x, a.l.x, b.h.x, b.l.x, r.h.x, r.l.x);
    df_add_lazy(a.h.y, a.l.y, b.h.y, b.l.y, r.h.y, r.l.y);
    return r;
}

__device__ __forceinline__ dfc df_csub(const dfc& a, const dfc& b)
{
    dfc r;
    df_add_lazy(a.h.x, a.l.x, -b.h.x, -b.l.x, r.h.x, r.l.x);
    df_add_lazy(a.h.y, a.l.y, -b.h.y, -b.l.y, r.h.y, r.l.y);
    return r;
}

// (a1 b1 - a2 b2) as a lazy pair: both products exact as (p, FMA residual),
// the cross terms with the lo words folded into the residual sum, and the
// difference of the two high products an error-free two_sum.  The lo * lo
// terms are dropped (below 2^-48 of the products; twiddles are normalised).
__device__ __forceinline__ void df_dot2_lazy(float a1h, float a1l, float b1h, float b1l, float a2h, float a2l,
                                             float b2h, float b2l, float& rh, float& rl)
{
    const float p1 = __fmul_rn(a1h, b1h);
    const float p2 = __fmul_rn(a2h, b2h);
    float t = __fsub_rn(fmaf(a1h, b1h, -p1), fmaf(a2h, b2h, -p2));
    t = fmaf(a1h, b1l, t);
    t = fmaf(a1l, b1h, t);
    t = fmaf(-a2h, b2l, t);
    t = fmaf(-a2l, b2h, t);
    float s, e;
    two_sum(p1, -p2, s, e);
    rh = s;
    rl = __fadd_rn(t, e);
}

__device__ __forceinline__ dfc df_cmul(const dfc& a, const dfc& w)
{
    dfc r;
    df_dot2_lazy(a.h.x, a.l.x, w.h.x, w.l.x, a.h.y, a.l.y, w.h.y, w.l.y, r.h.x, r.l.x);   // re
    df_dot2_lazy(a.h.x, a.l.x, w.h.y, w.l.y, -a.h.y, -a.l.y, w.h.x, w.l.x, r.h.y, r.l.y); // im
    return r;
}

// ------------------------------------------ register-staged radix-2 passes
// The radix-2 DIT transform of fft_stages (same twiddle values and
// per-butterfly arithmetic, float2 or float-float), but a thread loads the 2^K
// elements that K consecutive stages combine, runs those stages in registers
// and stores once: one shared-memory round trip and one __syncthreads per
// pass of up to 3 stages instead of per stage.  Lines are stored padded, one
// spare element per 8 (element e of a line at pad8(e), line length pad8(n)),
// which keeps the strided accesses of the first pass free of bank conflicts.
__device__ __host__ __forceinline__ int pad8(int e) { return e + (e >> 3); }

__device__ __forceinline__ void bfly(float2& a, float2& b, float2 w)
{
    const float2 t = cmul(b, w);
    const float2 u = a;
    a = cadd(u, t);
    b = csub(u, t);
}
__device__ __forceinline__ void bfly(dfc& a, dfc& b, const dfc& w)
{
    const dfc t = df_cmul(b, w);
    const dfc u = a;
    a = df_cadd(u, t);
    b = df_csub(u, t);
}
__device__ __forceinline__ float2 tw_conj(float2 w)
{
    w.y = -w.y;
    return w;
}
__device__ __forceinline__ dfc tw_conj(dfc w)
{
    w.h.y = -w.h.y;
    w.l.y = -w.l.y;
    return w;
}

// Butterflies with the twiddles 1 and -i (+i for the inverse): no multiply,
// the product by a unit is a swap and sign change of hi and lo parts.
__device__ __forceinline__ void bfly_one(float2& a, float2& b)
{
    const float2 u = a;
    a = cadd(u, b);
    b = csub(u, b);
}
__device__ __forceinline__ void bfly_one(dfc& a, dfc& b)
{
    const dfc u = a;
    a = df_cadd(u, b);
    b = df_csub(u, b);
}
__device__ __forceinline__ float2 mul_mi(float2 b, int sign) // b * (-i), or b * (+i) when sign > 0
{
    return sign > 0 ? make_float2(-b.y, b.x) : make_float2(b.y, -b.x);
}
__device__ __forceinline__ dfc mul_mi(const dfc& b, int sign)
{
    dfc r;
    r.h = mul_mi(b.h, sign);
    r.l = mul_mi(b.l, sign);
    return r;
}
template <typename C> __device__ __forceinline__ void bfly_mi(C& a, C& b, int sign)
{
    C t = mul_mi(b, sign);
    bfly_one(a, t);
    b = t;
}

// Stages s0+1 .. s0+K of an n = 2^logn DIT FFT on nl padded lines (stride ls).
// FIRST (s0 == 0): every twiddle index is known at compile time, and the
// twiddles 1 and -i (stages 1-3) skip the complex multiply.
template <int K, typename C, bool FIRST = false>
__device__ __forceinline__ void fft_pass(C* buf, int logn, int nl, int ls, const C* tw, int twlog, int sign, int s0)
{
    const int gsh = logn - K; // log2 of the groups per line
    const int ng = nl << gsh;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        const int line = g >> gsh, q = g & ((1 << gsh) - 1);
        const int j = q & ((1 << s0) - 1);
        const int base = ((q >> s0) << (s0 + K)) + j;
        C* L = buf + line * ls;
        C v[1 << K];
#pragma unroll
        for (int m = 0; m < (1 << K); ++m)
            v[m] = L[pad8(base + (m << s0))];
#pragma unroll
        for (int t = 1; t <= K; ++t) {
            const int hm = 1 << (t - 1);
#pragma unroll
            for (int m0 = 0; m0 < (1 << K); ++m0) {
                if (m0 & hm)
                    continue;
                const int k = m0 & (hm - 1); // twiddle exponent within the stage
                if (FIRST && k == 0) {
                    bfly_one(v[m0], v[m0 + hm]);                  // w = 1
                } else if (FIRST && 4 * k == (1 << t)) {
                    bfly_mi(v[m0], v[m0 + hm], sign);             // w = exp(-i pi/2)
                } else {
                    C w = tw[(1 << (s0 + t - 1)) - 1 + (k << s0) + j]; // stage-packed table
                    if (sign > 0)
                        w = tw_conj(w);
                    bfly(v[m0], v[m0 + hm], w);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < (1 << K); ++m)
            L[pad8(base + (m << s0))] = v[m];
    }
    __syncthreads();
}

// In-place DIT FFT of nl padded lines of length n = 2^logn (logn >= 3), input in
// bit-reversed order, in passes of at most 3 stages, twiddles from a
// stage-packed table (load_twiddles_packed).  Called by all threads.
template <typename C>
__device__ void fft_passes(C* buf, int logn, int nl, int ls, const C* tw, int twlog, int sign)
{
    const int np = (logn + 2) / 3;
    int s0 = 0;
    for (int p = 0; p < np; ++p) {
        const int k = (logn - s0 + (np - p) - 1) / (np - p);
        if (p == 0) {
            if (k == 3)
                fft_pass<3, C, true>(buf, logn, nl, ls, tw, twlog, sign, 0);
            else if (k == 2)
                fft_pass<2, C, true>(buf, logn, nl, ls, tw, twlog, sign, 0);
            else
                fft_pass<1, C, true>(buf, logn, nl, ls, tw, twlog, sign, 0);
        } else if (k == 3)
            fft_pass<3>(buf, logn, nl, ls, tw, twlog, sign, s0);
        else if (k == 2)
            fft_pass<2>(buf, logn, nl, ls, tw, twlog, sign, s0);
        else
            fft_pass<1>(buf, logn, nl, ls, tw, twlog, sign, s0);
        s0 += k;
    }
}

// Copies the twiddle table (2^(twlog-1) entries) into shared memory.
template <typename C>
__device__ void load_twiddles(C* dst, const C* src, int twlog)
{
    for (int k = threadIdx.x; k < (1 << (twlog - 1)); k += blockDim.x)
        dst[k] = src[k];
}

// Stage-packed twiddles for fft_passes of length 2^logn (2^logn - 1 entries):
// stage s keeps exp(-2 pi i k / 2^s), k < 2^(s-1), at (2^(s-1) - 1) + k, so the
// butterflies of a stage read consecutive entries (a table indexed k << (twlog
// - s) puts a warp's reads 2^(twlog-s) entries apart, in one bank).
template <typename C>
__device__ void load_twiddles_packed(C* dst, const C* src, int logn, int twlog)
{
    for (int i = threadIdx.x; i < (1 << logn) - 1; i += blockDim.x) {
        const int s = 32 - __clz(i + 1); // i + 1 in [2^(s-1), 2^s)
        const int k = i + 1 - (1 << (s - 1));
        dst[i] = src[k << (twlog - s)];
    }
}

// --------------------------------------------------- bispectrum element index
// Device replica of Bispectrum<T>::get_element's index path
// (include/bispectrum.h:482-512 with canonicalize_indices 553-589,
// classify_indices 162-174 and calc_offset 324-349), including the silent
// modulo-2^64 wrap of calc_offset.  Returns the packed offset or -1 where the
// reference throws std::out_of_range.  d: 4 sizes, 4 base sizes, min, max.
struct BispecDims {
    int sizes[4];
    int base[4];
    int mn[4];
    int mx[4];
    long long base_size;
};

__device__ __forceinline__ long long bispec_get_offset(const BispecDims& d, int i0, int i1, int i2, int i3, int* conj)
{
    if (abs(i2) > d.mx[2] || abs(i3) > d.mx[3]) {
        int t = i0; i0 = i2; i2 = t;
        t = i1; i1 = i3; i3 = t;
    }
    if (i0 < d.mn[0] || i0 > d.mx[0] || i1 < d.mn[1] || i1 > d.mx[1] || i2 < d.mn[2] || i2 > d.mx[2]
        || i3 < d.mn[3] || i3 > d.mx[3])
        return -1;
    int u0, u1, u2, u3, cj = 0;
    if (i0 <= 0 && i2 <= 0) { u0 = i0; u1 = i1; u2 = i2; u3 = i3; }
    else if (i0 > 0 && i2 > 0) { cj = 1; u0 = -i0; u1 = -i1; u2 = -i2; u3 = -i3; }
    else if (i0 > 0) {
        if (i0 + i2 > 0) { u0 = -i0 - i2; u1 = -i1 - i3; u2 = i2; u3 = i3; }
        else { cj = 1; u0 = -i0; u1 = -i1; u2 = i2 + i0; u3 = i3 + i1; }
    } else {
        if (i0 + i2 > 0) { u0 = i0; u1 = i1; u2 = -i2 - i0; u3 = -i3 - i1; }
        else { cj = 1; u0 = i0 + i2; u1 = i1 + i3; u2 = -i2; u3 = -i3; }
    }
    if (abs(u2) > d.mx[2] || abs(u3) > d.mx[3]) {
        int t = u0; u0 = u2; u2 = t;
        t = u1; u1 = u3; u3 = t;
    }
    int a0 = -u0, a1 = u1, a2 = -u2, a3 = u3;
    if (a0 < 0) a0 += d.sizes[0];
    if (a1 < 0) a1 += d.sizes[1];
    if (a2 < 0) a2 += d.sizes[2];
    if (a3 < 0) a3 += d.sizes[3];
    unsigned long long addr = (unsigned long long)(long long)a0;
    addr = addr * (unsigned long long)d.base[1] + (unsigned long long)(long long)a1;
    addr = addr * (unsigned long long)d.base[2] + (unsigned long long)(long long)a2;
    addr = addr * (unsigned long long)d.base[3] + (unsigned long long)(long long)a3;
    if (addr >= (unsigned long long)d.base_size)
        return -1;
    *conj = cj;
    return (long long)addr;
}

// ------------------------------------------------------ bounded device waits
// Every spin in these kernels is bounded by wall time (%globaltimer); on
// expiry the waiting thread records SMIP_DEV_ERR_TIMEOUT and gives up.
__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void record_error(int* err, int code)
{
    if (err)
        atomicCAS(err, 0, code);
}

// --------------------------------------------------------- mbarrier and TMA
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Invalidates a barrier whose phases are all complete, so that its memory
// can be initialised again (the persistent kernels reuse their rings).
__device__ __forceinline__ void mbar_inval(uint64_t* bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Non-blocking probe of the barrier phase with the given parity.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Waits for the barrier phase with the given parity; false after timeout_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t timeout_ns)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity))
                return true;
        if (globaltimer_ns() - t0 > timeout_ns)
            return false;
    }
}

// ------------------------------------------- thread-block clusters (DSMEM)
// A shared-memory variable of the CTA of rank `rank` in this CTA's cluster,
// as a shared::cluster address (mapa); valid for this CTA's own rank too.
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, uint32_t rank)
{
    uint32_t a;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(p)), "r"(rank));
    return a;
}
__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_size()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// acquire / release at cluster scope: pairs of them order the memory accesses
// (global and shared) of threads in different CTAs of the cluster
__device__ __forceinline__ int dsmem_ld_acquire(uint32_t a)
{
    int v;
    asm volatile("ld.acquire.cluster.shared::cluster.b32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ int dsmem_ld_relaxed(uint32_t a)
{
    int v;
    asm volatile("ld.relaxed.cluster.shared::cluster.b32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void dsmem_st_release(uint32_t a, int v)
{
    asm volatile("st.release.cluster.shared::cluster.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void dsmem_st_relaxed(uint32_t a, int v)
{
    asm volatile("st.relaxed.cluster.shared::cluster.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
// Stores into another CTA's shared memory that complete a transaction count
// on an mbarrier there (st.async): once the barrier's phase completes, a
// thread of that CTA that waited on it sees the data.
__device__ __forceinline__ void dsmem_st_async_f4(uint32_t a, float4 v, uint32_t bar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(a),
                 "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void dsmem_st_async_i(uint32_t a, int v, uint32_t bar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(a), "r"(v), "r"(bar)
                 : "memory");
}
// all threads of the cluster; every CTA's shared memory stays valid until
// all have arrived
__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// 3-D tiled TMA load into shared memory, completion signalled on bar.
__device__ __forceinline__ void tma_load_3d(void* dst, const void* tmap, int x, int y, int z, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
                     smem_u32(dst)),
                 "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
                 : "memory");
}

} // namespace smip_gpu
