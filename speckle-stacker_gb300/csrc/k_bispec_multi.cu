// k_bispec_multi.cu -- the bispectrum accumulation of many stacks' batches
// as one persistent launch (smip_batch_launch).  The unit of work is the
// single-stack kernel's (k_bispec.cuh), so results are bit-identical.
#include <cstring>
#include <vector>

#include "k_bispec.cuh"

namespace smip_gpu {

// ------------------------------------------- many stacks, one launch
// A persistent grid (one CTA per SM) takes units from a device work list of
// (stack, unit) pairs -- every stack's tiles and split-tile parts, exactly the
// units its own launch would run, longest first -- so the bispectrum work of
// stacks of any sizes and depths runs as one launch.  Each unit is the
// single-stack kernel's unit (same tile decomposition, same split parts
// merged in part order), so every stack's result is bit-identical to its own
// launch.  Per stack the record below holds its three tensor maps over its
// spectra and its launch arguments; records, work list and counter live in
// device memory, so the launch itself never changes.
struct MultiStackRec {
    CUtensorMap m[3];
    BispecArgs a;
    int de;    // kernel depth class (a multiple of 8)
    int exact; // the stack's depth is de itself
};

template <int DE> struct MaxSmem {
    static constexpr int v = BCfg<DE>::SMEM > MaxSmem<DE - 8>::v ? BCfg<DE>::SMEM : MaxSmem<DE - 8>::v;
};
template <> struct MaxSmem<0> {
    static constexpr int v = 0;
};
constexpr int kMultiSmem = MaxSmem<64>::v;

// One unit as a separate function per depth class, so that each keeps the
// register allocation of its own kernel inside the dispatching loop.
template <int DE, bool EXACT>
__device__ __noinline__ bool bispec_unit_call(unsigned char* smem, const MultiStackRec* r, int unit)
{
    return bispec_unit<DE, EXACT>(smem, &r->m[0], &r->m[1], &r->m[2], r->a, unit);
}

// ctrl[0]: work items; ctrl[1]: next item (zero at launch)
__global__ void __launch_bounds__(512, 1) bispec_multi_kernel(const MultiStackRec* __restrict__ recs,
                                                              const int2* __restrict__ items, int* ctrl)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_item;
    const int nitems = *reinterpret_cast<volatile int*>(ctrl);
    const int lane = threadIdx.x & 31;
    for (;;) {
        __syncthreads(); // every thread has read s_item
        if (threadIdx.x == 0)
            s_item = atomicAdd(&ctrl[1], 1);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems)
            break;
        const int2 w = items[it];
        const MultiStackRec* r = recs + w.x;
        if (lane == 0) // the ring's issuers: lane 0 of any warp
            for (int k = 0; k < 3; ++k)
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(&r->m[k]) : "memory");
        bool ok = true;
        switch (r->de * 2 + r->exact) {
#define SMIP_MULTI_CASE(DE)                                                                                       \
    case 2 * DE + 1: ok = bispec_unit_call<DE, true>(smem, r, w.y); break;                                        \
    case 2 * DE: ok = bispec_unit_call<DE, false>(smem, r, w.y); break;
            SMIP_MULTI_CASE(8) SMIP_MULTI_CASE(16) SMIP_MULTI_CASE(24) SMIP_MULTI_CASE(32)
            SMIP_MULTI_CASE(40) SMIP_MULTI_CASE(48) SMIP_MULTI_CASE(56) SMIP_MULTI_CASE(64)
#undef SMIP_MULTI_CASE
        default: break;
        }
        if (!__syncthreads_and(ok)) // a wait expired (recorded in the stack's error word): stop
            break;
    }
}

size_t bispec_multi_rec_bytes() { return sizeof(MultiStackRec); }

int bispec_multi_fill(void* rec, const BispecLaunch& L, const Geometry& g, std::vector<int>* unit_frames)
{
    MultiStackRec r; // 64-byte aligned here, as the tensor-map encoder requires; copied out at the end
    std::memset(&r, 0, sizeof r);
    const int de = (g.De + 7) / 8 * 8;
    r.de = de;
    r.exact = g.De % 8 == 0;
    bool ok = false;
    switch (de) {
#define SMIP_MULTI_FILL(DE)                                                                                       \
    case DE: ok = make_maps<DE>(r.m, L, g); r.a = fill_args<DE>(L, g); break;
        SMIP_MULTI_FILL(8) SMIP_MULTI_FILL(16) SMIP_MULTI_FILL(24) SMIP_MULTI_FILL(32)
        SMIP_MULTI_FILL(40) SMIP_MULTI_FILL(48) SMIP_MULTI_FILL(56) SMIP_MULTI_FILL(64)
#undef SMIP_MULTI_FILL
    default: return -1;
    }
    if (!ok)
        return -1;
    // frames per unit: whole tiles take the batch, split units their part
    const int units = r.a.nfull + r.a.nsplit;
    unit_frames->resize(units);
    for (int u = 0; u < units; ++u) {
        if (u < r.a.nfull) {
            (*unit_frames)[u] = L.nframes;
        } else {
            const int part = (u - r.a.nfull) % r.a.P;
            (*unit_frames)[u] = (int)((long long)(part + 1) * L.nframes / r.a.P - (long long)part * L.nframes / r.a.P);
        }
    }
    std::memcpy(rec, &r, sizeof r);
    return units;
}

cudaError_t launch_bispec_multi(const void* recs, const int2* items, int* ctrl, int num_sms, cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(bispec_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMultiSmem);
    if (e != cudaSuccess)
        return e;
    bispec_multi_kernel<<<num_sms, 512, kMultiSmem, st>>>(static_cast<const MultiStackRec*>(recs), items, ctrl);
    note_launches(1);
    return cudaGetLastError();
}

} // namespace smip_gpu
