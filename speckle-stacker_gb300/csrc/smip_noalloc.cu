// smip_noalloc.cu -- integer shift of a frame against a reference frame
// without any device-memory allocation.
//
// Who needs this: callers that must not allocate device memory once they are
// running.  Examples are acquisition loops that register their buffers at
// start-up and keep a fixed frame cadence, where a cudaMalloc can stall the
// device, and plug-ins inside applications whose device memory belongs to the
// host's pool allocator, where a direct cudaMalloc escapes the pool's budget
// and accounting.  Such callers pass device pointers for the inputs and the
// output, and every intermediate buffer lives in the fixed array below.
//
// The array is a file-scope __device__ object of kScratchBytes (about 3 MB,
// enough for frames up to 256 x 256).  Host code may not use its name as an
// address, so each call looks the address up with cudaGetSymbolAddress (with
// the caller's device current; a lookup allocates nothing once the array is
// resident).  The first call on a device does the set-up: the lookup makes
// the CUDA runtime load this library's module and place the array on the
// device (CUDA loads modules lazily by default, so this is where the array's
// memory is taken), the FFT twiddle tables are copied into it, and one
// 16 x 16 warm-up shift runs every kernel the call uses, so that their
// modules are loaded too.  That first call therefore allocates and must come
// at start-up, before any stream capture; later calls allocate nothing.  A
// device reset (cudaDeviceReset) discards the array: the next call sees a
// new address and repeats the set-up, so it allocates again.
//
// All calls on a device share the array: two calls whose work overlaps on
// the GPU race with each other and must be ordered by the caller (one
// stream, or events).  Each call writes every scratch region before it reads
// it, so the contents left by an earlier call never matter.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/smip_gpu.h"
#include "smip_internal.h"

using namespace smip_gpu;

namespace {

constexpr int kMaxN = 256;                                   // largest ncols / nrows
constexpr size_t kHalf = (size_t)(kMaxN / 2 + 1) * kMaxN;    // half-plane elements
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffGt = 0;                                             // 2 frames, float-float
constexpr size_t kOffS = kOffGt + align256(2 * kHalf * sizeof(dfc));     // 1 frame
constexpr size_t kOffT = kOffS + align256(kHalf * sizeof(float2));       // 1 frame
constexpr size_t kOffR = kOffT + align256(kHalf * sizeof(float2));       // reference spectrum
constexpr size_t kOffP = kOffR + align256(kHalf * sizeof(float2));       // power partials
constexpr size_t kOffC = kOffP + align256(kHalf * sizeof(double));       // correlation
constexpr size_t kOffM = kOffC + align256((size_t)kMaxN * kMaxN * sizeof(float)); // row maxima
constexpr size_t kOffQ = kOffM + align256((size_t)kMaxN * sizeof(float));          // sum of squares
constexpr int kTw = 1 << (kTwLog - 1);
constexpr size_t kOffTw = kOffQ + 256;                                   // FP32 twiddles
constexpr size_t kOffTwDf = kOffTw + align256(kTw * sizeof(float2));     // float-float twiddles
constexpr size_t kOffWarm = kOffTwDf + align256(kTw * sizeof(dfc));     // warm-up frame (16 x 16 doubles, zero)
constexpr size_t kWarmN = 16;
constexpr size_t kOffWarmOut = kOffWarm + align256(kWarmN * kWarmN * sizeof(double)); // warm-up shift
constexpr size_t kScratchBytes = kOffWarmOut + 256;

static __device__ __align__(256) unsigned char g_xcorr_scratch[kScratchBytes];

std::mutex g_mu;
std::vector<unsigned char*> g_base; // per device: the array's address when it was set up

int fail(int code, const std::string& m)
{
    set_error_message(m);
    return code;
}

bool pow2_in(long v);
int ilog2i(long v);
cudaError_t run_shift(unsigned char* base, const double* ref, const double* frame, long ncols, long nrows, int* shift,
                      cudaStream_t st);

// With the caller's device current: look up the array's device address and,
// when it is new for this device (first call, or after a device reset), fill
// the twiddle tables and run one warm-up shift on a zero 16 x 16 frame held
// in the array, which loads every kernel this entry point launches.
int setup(int dev, cudaStream_t st, unsigned char** base)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_base.size() <= dev)
        g_base.resize(dev + 1, nullptr);
    unsigned char* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_xcorr_scratch);
    if (e != cudaSuccess)
        return fail(SMIP_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    if (g_base[dev] != p) {
        std::vector<float2> t32(kTw);
        std::vector<dfc> tdf(kTw);
        for (int k = 0; k < kTw; ++k) {
            const double a = 2.0 * M_PI * (double)k / (double)(1 << kTwLog);
            const double c = std::cos(a), s = -std::sin(a);
            t32[k] = make_float2((float)c, (float)s);
            tdf[k].h = t32[k];
            tdf[k].l = make_float2((float)(c - (double)t32[k].x), (float)(s - (double)t32[k].y));
        }
        e = cudaMemcpy(p + kOffTw, t32.data(), sizeof(float2) * kTw, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(p + kOffTwDf, tdf.data(), sizeof(dfc) * kTw, cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            return fail(SMIP_E_CUDA, std::string("twiddle upload: ") + cudaGetErrorString(e));
        const double* warm = reinterpret_cast<const double*>(p + kOffWarm);
        e = cudaMemsetAsync(p + kOffWarm, 0, kWarmN * kWarmN * sizeof(double), st);
        if (e == cudaSuccess)
            e = run_shift(p, warm, warm, kWarmN, kWarmN, reinterpret_cast<int*>(p + kOffWarmOut), st);
        if (e != cudaSuccess)
            return fail(SMIP_E_CUDA, std::string("warm-up shift: ") + cudaGetErrorString(e));
        g_base[dev] = p;
    }
    *base = p;
    return SMIP_OK;
}

bool pow2_in(long v) { return v >= 16 && v <= kMaxN && (v & (v - 1)) == 0; }

int ilog2i(long v)
{
    int l = 0;
    while ((1L << l) < v)
        ++l;
    return l;
}

// The shift's kernels on stream st, every intermediate inside the array at base.
cudaError_t run_shift(unsigned char* base, const double* ref, const double* frame, long ncols, long nrows, int* shift,
                      cudaStream_t st)
{
    Geometry g {};
    g.W = (int)ncols;
    g.H = (int)nrows;
    g.logW = ilog2i(ncols);
    g.logH = ilog2i(nrows);
    g.hw = (int)ncols / 2 + 1;
    const size_t half = (size_t)g.hw * g.H;
    dfc* Gt = reinterpret_cast<dfc*>(base + kOffGt);
    float2* S = reinterpret_cast<float2*>(base + kOffS);
    float2* T = reinterpret_cast<float2*>(base + kOffT);
    float2* R = reinterpret_cast<float2*>(base + kOffR);
    double* Pp = reinterpret_cast<double*>(base + kOffP);
    float* corr = reinterpret_cast<float*>(base + kOffC);
    float* rowmax = reinterpret_cast<float*>(base + kOffM);
    double* refsq = reinterpret_cast<double*>(base + kOffQ);
    const float2* tw = reinterpret_cast<const float2*>(base + kOffTw);
    const dfc* twdf = reinterpret_cast<const dfc*>(base + kOffTwDf);
    const long long n = (long long)ncols * nrows;
    cudaError_t e = launch_sumsq(SMIP_F64, ref, n, refsq, st);
    if (e == cudaSuccess) e = launch_row_pass(SMIP_F64, ref, n, 1, g, Gt, twdf, st);
    if (e == cudaSuccess) e = launch_row_pass(SMIP_F64, frame, n, 1, g, Gt + half, twdf, st);
    if (e == cudaSuccess) e = launch_col_pass(1, Gt, S, R, R, T, Pp, 1, 16, 0, g, twdf, tw, st);
    if (e == cudaSuccess) e = launch_col_pass(0, Gt + half, S, R, nullptr, T, Pp, 1, 16, 0, g, twdf, tw, st);
    if (e == cudaSuccess) e = launch_xcorr_rows(T, corr, rowmax, 1, g, tw, st);
    if (e == cudaSuccess) e = launch_xcorr_shift(SMIP_F64, corr, rowmax, frame, n, ref, refsq, 1, 0, g, shift, st);
    return e;
}

} // namespace

extern "C" int smip_xcorr_displacement_noalloc(const double* ref, const double* frame, long ncols, long nrows,
                                               int* shift, void* stream)
{
    if (!ref || !frame || !shift)
        return fail(SMIP_E_INVALID_ARGUMENT, "null device pointer");
    if (!pow2_in(ncols) || !pow2_in(nrows))
        return fail(SMIP_E_UNSUPPORTED, "smip_xcorr_displacement_noalloc: ncols and nrows must be powers of two in "
                                        "[16, 256] (the fixed scratch array holds frames up to 256 x 256)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return fail(SMIP_E_CUDA, "cudaGetDevice failed");
    unsigned char* base = nullptr;
    int rc = setup(dev, static_cast<cudaStream_t>(stream), &base);
    if (rc)
        return rc;
    cudaError_t e = run_shift(base, ref, frame, ncols, nrows, shift, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return fail(SMIP_E_CUDA, cudaGetErrorString(e));
    return SMIP_OK;
}
