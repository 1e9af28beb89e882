// k_fft.cu -- per-frame forward FFT, power spectrum and the
// cross-correlation transforms.
//
// Replaces the FFTW calls of smip-cli/main.cpp:256-259, 271, 296 (forward
// c2c of each frame, FP64 in the reference), the |F|^2 accumulation of
// main.cpp:274-279, 300-305 and the r2c / c2r pair of
// CrossCorrelation::correlate (include/crosscorrel.h:103-141).  Frames are
// real, so only the u_x <= 0 half plane is computed; the other half is its
// complex conjugate mirror.
//
// Precision.  The forward transform runs in float-float arithmetic (~44-bit,
// smip_dev.cuh) on the FP32 pipes and is rounded to FP32 once at the end, so
// every frequency bin -- including bins 10^4 x weaker than the frame's
// energy -- carries FP32 relative accuracy, as the reference's FP64 FFT
// narrowed to complex<float> (bispectrum.h:399) does.  A plain FP32 FFT loses
// up to 1e-2 relative accuracy in such bins and 5e-2 in bispectrum elements
// that are cancellations of them.  The power spectrum is |F|^2 of the
// float-float values, summed over a chunk's frames in float-float and over
// chunks in FP64.  The correlation's inverse transform only
// locates the peak (candidates are re-scored exactly, k_xcorr.cu) and stays
// FP32.
//
// Layout written for the bispectrum kernel (per frame, float2):
//   S[a][c] = F(x = -a, y = c - H/2),  a in [0, W/2], c in [0, H)
// i.e. rows indexed by -u_x (the reference's packed dim 0, bispectrum.h:327)
// and y centred, so every tile the bispectrum kernel needs is one rectangular
// TMA box, with zero fill exactly where the reference's loop bounds stop
// (bispectrum.h:397-398).
#include "smip_dev.cuh"

namespace smip_gpu {

template <typename T> __device__ __forceinline__ float2 pix_df(const T* p, long long i)
{
    return make_float2((float)p[i], 0.f); // u8/u16/f32 are exact in FP32
}
template <> __device__ __forceinline__ float2 pix_df<double>(const double* p, long long i)
{
    const double v = p[i];
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

__device__ __forceinline__ float2 df_round(const dfc& v) { return make_float2(v.h.x + v.l.x, v.h.y + v.l.y); }

// ---------------------------------------------------------------- row pass
// Two real rows per complex FFT of length W (x0 + i x1), float-float; the
// half-spectra are separated afterwards.  Output G'(a, y) = sum_x f(x, y)
// exp(+2 pi i a x / W), float-float, stored [f][a][y].
// copy_out (optional): the frames as read, written to device memory [f][y][x]
// with the same stride -- the batch's frame buffer when the frames are read
// straight from mapped page-locked host memory.
template <typename T>
__global__ void __launch_bounds__(256, 4) row_pass_kernel(const T* __restrict__ frames, long long fstride, int logW, int H,
                                                        int hw, dfc* __restrict__ Gt, const dfc* __restrict__ tw_g,
                                                        T* __restrict__ copy_out)
{
    extern __shared__ dfc smdf[];
    const int W = 1 << logW;
    dfc* tw = smdf;                                // W - 1, stage-packed (+1 spare)
    dfc* lines = smdf + W;                         // [kRowBlock/2][pad8(W) + 1]
    // one spare element per line: the output pass reads the same element of
    // the 8 lines in one warp, which a 128-byte multiple would put in one bank
    const int LW = pad8(W) + 1;
    const int f = blockIdx.y;
    const int y0 = blockIdx.x * kRowBlock;
    const T* fr = frames + (long long)f * fstride + (long long)y0 * W;
    T* co = copy_out ? copy_out + (long long)f * fstride + (long long)y0 * W : nullptr;
    load_twiddles_packed(tw, tw_g, logW, kTwLog);
    auto put = [&](int idx, float2 v) {
        const int r = idx >> logW, x = idx & (W - 1);
        dfc& d = lines[(r >> 1) * LW + pad8(bitrev(x, logW))];
        if (r & 1) {
            d.h.y = v.x;
            d.l.y = v.y;
        } else {
            d.h.x = v.x;
            d.l.x = v.y;
        }
    };
    // 16-byte loads (16, 8 or 4 pixels; W >= 16 keeps a vector inside one
    // row) of both rows of a line, stored as whole complex values: a warp's
    // stores of one vector element go to 32 bit-reversed slots that the
    // padding spreads over all banks
    constexpr int PV = sizeof(T) <= 4 ? 16 / (int)sizeof(T) : 1;
    if (PV > 1 && (reinterpret_cast<uintptr_t>(fr) & 15) == 0 && (reinterpret_cast<uintptr_t>(co) & 15) == 0) {
        const int vpl = W / PV; // vectors per row
        for (int i = threadIdx.x; i < (kRowBlock / 2) * vpl; i += blockDim.x) {
            const int pr = i / vpl, x0 = (i - pr * vpl) * PV;
            T p0[PV], p1[PV];
            *reinterpret_cast<uint4*>(p0) = *reinterpret_cast<const uint4*>(fr + (2 * pr) * W + x0);
            *reinterpret_cast<uint4*>(p1) = *reinterpret_cast<const uint4*>(fr + (2 * pr + 1) * W + x0);
            if (co) {
                *reinterpret_cast<uint4*>(co + (2 * pr) * W + x0) = *reinterpret_cast<const uint4*>(p0);
                *reinterpret_cast<uint4*>(co + (2 * pr + 1) * W + x0) = *reinterpret_cast<const uint4*>(p1);
            }
            dfc* L = lines + pr * LW;
#pragma unroll
            for (int e = 0; e < PV; ++e) {
                dfc d;
                d.h = make_float2((float)p0[e], (float)p1[e]);
                d.l = make_float2(0.f, 0.f);
                L[pad8(bitrev(x0 + e, logW))] = d;
            }
        }
    } else {
        for (int idx = threadIdx.x; idx < kRowBlock * W; idx += blockDim.x) {
            put(idx, pix_df(fr, idx));
            if (co)
                co[idx] = fr[idx];
        }
    }
    __syncthreads();
    fft_passes(lines, logW, kRowBlock / 2, LW, tw, kTwLog, -1);
    dfc* out = Gt + (long long)f * hw * H;
    for (int idx = threadIdx.x; idx < hw * kRowBlock; idx += blockDim.x) {
        const int a = idx / kRowBlock, r = idx - a * kRowBlock;
        const dfc* Z = lines + (r >> 1) * LW;
        const dfc za = Z[pad8(a)], zb = Z[pad8((W - a) & (W - 1))];
        dfc g;
        if ((r & 1) == 0) { // conj of X0 = (Z(a) + conj Z(-a)) / 2
            df_add_lazy(za.h.x, za.l.x, zb.h.x, zb.l.x, g.h.x, g.l.x);
            df_add_lazy(zb.h.y, zb.l.y, -za.h.y, -za.l.y, g.h.y, g.l.y);
        } else { // conj of X1 = (Z(a) - conj Z(-a)) / 2i
            df_add_lazy(za.h.y, za.l.y, zb.h.y, zb.l.y, g.h.x, g.l.x);
            df_add_lazy(za.h.x, za.l.x, -zb.h.x, -zb.l.x, g.h.y, g.l.y);
        }
        g.h.x *= 0.5f; g.l.x *= 0.5f; g.h.y *= 0.5f; g.l.y *= 0.5f;
        out[(long long)a * H + y0 + r] = g;
    }
}

// ------------------------------------------------------------- column pass
// One CTA per (a, chunk of frames).  Float-float forward FFT along y gives
// Fm(a, y) = F(-a, y); writes S (rounded to FP32), accumulates |F|^2 in float-float
// (frame order), and for the correlation computes the FP32 inverse
// y-transform of conj(R) * Fm into T.
__global__ void __launch_bounds__(256) col_pass_kernel(int mode, const dfc* __restrict__ Gt, float2* __restrict__ S,
                                                        const float2* __restrict__ Rbuf, float2* __restrict__ Rout,
                                                        float2* __restrict__ T, double* __restrict__ Ppart,
                                                        int nframes, int fpc, int skip_xcorr_frame0, int logH, int hw,
                                                        const dfc* __restrict__ twdf_g, const float2* __restrict__ tw_g)
{
    extern __shared__ dfc smdf[];
    const int H = 1 << logH;
    dfc* twd = smdf;                                               // H - 1, stage-packed (+1 spare)
    const int LH = pad8(H);                                        // padded line length
    dfc* L1 = twd + H;                                             // [kColLines][LH]
    float2* tw = reinterpret_cast<float2*>(L1 + kColLines * LH);   // H - 1, stage-packed (+1 spare)
    float2* R = tw + H;                                            // [H]
    float2* L2 = R + H;                                            // [kColLines][LH]
    float2* pacc = reinterpret_cast<float2*>(L2 + kColLines * LH); // [H] float-float (hi, lo)
    const int a = blockIdx.x;
    const int chunk = blockIdx.y;
    const int fbeg = chunk * fpc;
    const int fend = min(nframes, fbeg + fpc);
    const long long gstride = (long long)hw * H;
    load_twiddles_packed(twd, twdf_g, logH, kTwLog);
    load_twiddles_packed(tw, tw_g, logH, kTwLog);
    if (mode == 0)
        for (int y = threadIdx.x; y < H; y += blockDim.x) {
            R[y] = Rbuf[(long long)a * H + y];
            pacc[y] = make_float2(0.f, 0.f);
        }
    for (int f0 = fbeg; f0 < fend; f0 += kColLines) {
        const int nl = min(kColLines, fend - f0);
        __syncthreads();
        // eight consecutive y per thread: a warp's stores of one of them go to
        // 32 bit-reversed slots that the padding spreads over all banks
        for (int i = threadIdx.x; i < nl * (H / 8); i += blockDim.x) {
            const int l = i / (H / 8), y0 = (i - l * (H / 8)) * 8;
            const dfc* src = Gt + (f0 + l) * gstride + (long long)a * H + y0;
            dfc* L = L1 + l * LH;
#pragma unroll
            for (int e = 0; e < 8; ++e)
                L[pad8(bitrev(y0 + e, logH))] = src[e];
        }
        __syncthreads();
        fft_passes(L1, logH, nl, LH, twd, kTwLog, -1);
        if (mode == 1) { // reference spectrum only
            for (int y = threadIdx.x; y < H; y += blockDim.x)
                Rout[(long long)a * H + y] = df_round(L1[pad8(y)]);
            return;
        }
        for (int idx = threadIdx.x; idx < nl * H; idx += blockDim.x) {
            const int l = idx >> logH, c = idx & (H - 1);
            S[(f0 + l) * gstride + (long long)a * H + c] = df_round(L1[l * LH + pad8((c + H / 2) & (H - 1))]);
        }
        // power spectrum, frames in order per element: |F|^2 of the float-float values
        // summed in float-float (~48-bit) on the FP32 pipes; GB300's FP64 rate is
        // too low for this per-element sum
        for (int c = threadIdx.x; c < H; c += blockDim.x) {
            float ah = pacc[c].x, al = pacc[c].y;
            for (int l = 0; l < nl; ++l) {
                dfc v = L1[l * LH + pad8((c + H / 2) & (H - 1))];
                df_norm(v.h.x, v.l.x); // the FFT leaves lazy pairs
                df_norm(v.h.y, v.l.y);
                float rh, rl, ih, il, sh, sl;
                df_mul(v.h.x, v.l.x, v.h.x, v.l.x, rh, rl);
                df_mul(v.h.y, v.l.y, v.h.y, v.l.y, ih, il);
                df_add(rh, rl, ih, il, sh, sl);
                df_add(ah, al, sh, sl, ah, al);
            }
            pacc[c] = make_float2(ah, al);
        }
        // correlation product conj(R) * F in FP32, bit-reversed for the inverse FFT
        for (int idx = threadIdx.x; idx < nl * H; idx += blockDim.x) {
            const int l = idx >> logH, y = idx & (H - 1);
            const float2 r = R[y], v = df_round(L1[l * LH + pad8(y)]);
            L2[l * LH + pad8(bitrev(y, logH))] = make_float2(r.x * v.x + r.y * v.y, r.x * v.y - r.y * v.x);
        }
        __syncthreads();
        fft_passes(L2, logH, nl, LH, tw, kTwLog, +1);
        for (int idx = threadIdx.x; idx < nl * H; idx += blockDim.x) {
            const int l = idx >> logH, y = idx & (H - 1);
            if (skip_xcorr_frame0 && f0 + l == 0)
                continue;
            T[(f0 + l) * gstride + (long long)a * H + y] = L2[l * LH + pad8(y)];
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < H; c += blockDim.x)
        Ppart[(long long)chunk * gstride + (long long)a * H + c] = (double)pacc[c].x + (double)pacc[c].y;
}

__global__ void power_reduce_kernel(double* __restrict__ P, const double* __restrict__ Ppart, int nchunks, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double acc = P[i];
        for (int c = 0; c < nchunks; ++c)
            acc += Ppart[(long long)c * n + i];
        P[i] = acc;
    }
}

// ------------------------------------------------------- correlation rows
// c2r along x of T(-a, y): Hermitian extension Z(k) = T(a=k)* for 0<k<W/2,
// T(a=W-k) for k>W/2, real parts at k = 0, W/2 (as FFTW's c2r ignores those
// imaginary parts); two rows per complex FFT.  Output: unnormalised
// correlation c[y][x] = W*H * sum ref(p) frame(p + (x,y)).
__global__ void __launch_bounds__(256) xcorr_rows_kernel(const float2* __restrict__ Gt, float* __restrict__ corr,
                                                          float* __restrict__ rowmax, int logW, int H, int hw,
                                                          const float2* __restrict__ tw_g)
{
    extern __shared__ float2 sm[];
    const int W = 1 << logW;
    // Ts rows padded to kRowBlock + 1: the Hermitian build below reads one
    // column r of consecutive a per warp, which an unpadded 128-byte row
    // stride would put in one bank pair
    constexpr int TS = kRowBlock + 1;
    float2* tw = sm;                               // W - 1, stage-packed (+1 spare)
    float2* Ts = tw + W;                           // [hw][TS]
    float2* lines = Ts + hw * TS;                  // [kRowBlock/2][pad8(W)]
    const int LW = pad8(W);
    const int f = blockIdx.y;
    const int y0 = blockIdx.x * kRowBlock;
    const float2* T = Gt + (long long)f * hw * H;
    load_twiddles_packed(tw, tw_g, logW, kTwLog);
    for (int idx = threadIdx.x; idx < hw * kRowBlock; idx += blockDim.x) {
        const int a = idx / kRowBlock, r = idx - a * kRowBlock;
        Ts[a * TS + r] = T[(long long)a * H + y0 + r];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < (kRowBlock / 2) * W; idx += blockDim.x) {
        const int p = idx >> logW, k = idx & (W - 1);
        float2 z[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = 2 * p + h;
            if (k == 0)
                z[h] = make_float2(Ts[r].x, 0.f);
            else if (k < W / 2)
                z[h] = cconj(Ts[k * TS + r]);
            else if (k == W / 2)
                z[h] = make_float2(Ts[(W / 2) * TS + r].x, 0.f);
            else
                z[h] = Ts[(W - k) * TS + r];
        }
        lines[p * LW + pad8(bitrev(k, logW))] = make_float2(z[0].x - z[1].y, z[0].y + z[1].x);
    }
    __syncthreads();
    fft_passes(lines, logW, kRowBlock / 2, LW, tw, kTwLog, +1);
    float* out = corr + (long long)f * W * H + (long long)y0 * W;
    for (int idx = threadIdx.x; idx < kRowBlock * W; idx += blockDim.x) {
        const int r = idx >> logW, x = idx & (W - 1);
        const float2 v = lines[(r >> 1) * LW + pad8(x)];
        out[idx] = (r & 1) ? v.y : v.x;
    }
    // every row's maximum (16 threads per row), so that the peak search reads
    // the rows that can hold candidates only
    static_assert(kRowBlock * 16 == 256, "16 threads per row");
    const int r = threadIdx.x >> 4, sub = threadIdx.x & 15;
    const float2* Lr = lines + (r >> 1) * LW;
    float m = -INFINITY;
    for (int x = sub; x < W; x += 16) {
        const float2 v = Lr[pad8(x)];
        m = fmaxf(m, (r & 1) ? v.y : v.x);
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (sub == 0)
        rowmax[(long long)f * H + y0 + r] = m;
}

// ----------------------------------------------------- spectrum import
// FFT-order complex<double> spectra (ncols x nrows) -> S layout (float2).
// S rows have pitch Hs >= H.
__global__ void import_spectra_kernel(const double2* __restrict__ in, int nframes, int W, int H, int Hs, int hw,
                                      float2* __restrict__ S)
{
    const long long per = (long long)hw * H;
    const long long n = per * nframes;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long f = i / per;
        const int rem = (int)(i - f * per);
        const int a = rem / H, c = rem - a * H;
        const int x = a == 0 ? 0 : W - a;   // x = -a
        int y = c + (H - H / 2);            // y = c - H/2, wrapped
        y -= y >= H ? H : 0;
        const double2 v = in[f * (long long)W * H + (long long)y * W + x];
        S[(f * hw + a) * (long long)Hs + c] = make_float2((float)v.x, (float)v.y);
    }
}

// ------------------------------------------------------------- launchers
static int grid_for(long long n, int block)
{
    long long g = (n + block - 1) / block;
    return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

// The kernels' dynamic shared memory limit is set to their largest size over
// every supported frame size (2^kMaxLog per axis), not to this launch's: the
// attribute is per function, so concurrent launches of different shapes from
// several host threads would otherwise lower it under each other's launches.
template <typename K> static cudaError_t allow_smem(K kern, size_t max_smem)
{
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
}
static size_t row_pass_smem(int W) { return sizeof(dfc) * (W + (kRowBlock / 2) * (pad8(W) + 1)); }
static size_t col_pass_smem(int H)
{
    return sizeof(dfc) * (H + kColLines * pad8(H)) + sizeof(float2) * (H + H + kColLines * pad8(H)) + sizeof(double) * H;
}
static size_t xcorr_rows_smem(int W) { return sizeof(float2) * (W + (W / 2 + 1) * (kRowBlock + 1) + (kRowBlock / 2) * pad8(W)); }

cudaError_t launch_row_pass(int dtype, const void* frames, long long fstride, int nframes, const Geometry& g, dfc* Gt,
                            const dfc* twdf, cudaStream_t st, void* copy_out)
{
    const dim3 grid(g.H / kRowBlock, nframes);
    const size_t smem = row_pass_smem(g.W), smem_max = row_pass_smem(1 << kMaxLog);
    cudaError_t e = cudaSuccess;
    switch (dtype) {
    case 0:
        if ((e = allow_smem(row_pass_kernel<uint8_t>, smem_max)) != cudaSuccess) return e;
        row_pass_kernel<uint8_t><<<grid, 256, smem, st>>>((const uint8_t*)frames, fstride, g.logW, g.H, g.hw, Gt, twdf,
                                                          (uint8_t*)copy_out);
        break;
    case 1:
        if ((e = allow_smem(row_pass_kernel<uint16_t>, smem_max)) != cudaSuccess) return e;
        row_pass_kernel<uint16_t><<<grid, 256, smem, st>>>((const uint16_t*)frames, fstride, g.logW, g.H, g.hw, Gt, twdf,
                                                           (uint16_t*)copy_out);
        break;
    case 2:
        if ((e = allow_smem(row_pass_kernel<float>, smem_max)) != cudaSuccess) return e;
        row_pass_kernel<float><<<grid, 256, smem, st>>>((const float*)frames, fstride, g.logW, g.H, g.hw, Gt, twdf,
                                                        (float*)copy_out);
        break;
    default:
        if ((e = allow_smem(row_pass_kernel<double>, smem_max)) != cudaSuccess) return e;
        row_pass_kernel<double><<<grid, 256, smem, st>>>((const double*)frames, fstride, g.logW, g.H, g.hw, Gt, twdf,
                                                         (double*)copy_out);
        break;
    }
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_col_pass(int mode, const dfc* Gt, float2* S, const float2* Rbuf, float2* Rout, float2* T,
                            double* Ppart, int nframes, int fpc, int skip_xcorr_frame0, const Geometry& g,
                            const dfc* twdf, const float2* tw, cudaStream_t st)
{
    const int nchunks = mode == 1 ? 1 : (nframes + fpc - 1) / fpc;
    const dim3 grid(g.hw, nchunks);
    const size_t smem = col_pass_smem(g.H);
    cudaError_t e = allow_smem(col_pass_kernel, col_pass_smem(1 << kMaxLog));
    if (e != cudaSuccess)
        return e;
    col_pass_kernel<<<grid, 256, smem, st>>>(mode, Gt, S, Rbuf, Rout, T, Ppart, mode == 1 ? 1 : nframes, fpc,
                                             skip_xcorr_frame0, g.logH, g.hw, twdf, tw);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_power_reduce(double* P, const double* Ppart, int nchunks, const Geometry& g, cudaStream_t st)
{
    const long long n = (long long)g.hw * g.H;
    power_reduce_kernel<<<grid_for(n, 256), 256, 0, st>>>(P, Ppart, nchunks, n);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_xcorr_rows(const float2* T, float* corr, float* rowmax, int nframes, const Geometry& g,
                              const float2* tw, cudaStream_t st)
{
    const dim3 grid(g.H / kRowBlock, nframes);
    const size_t smem = xcorr_rows_smem(g.W);
    cudaError_t e = allow_smem(xcorr_rows_kernel, xcorr_rows_smem(1 << kMaxLog));
    if (e != cudaSuccess)
        return e;
    xcorr_rows_kernel<<<grid, 256, smem, st>>>(T, corr, rowmax, g.logW, g.H, g.hw, tw);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_import_spectra(const double* spectra, int nframes, const Geometry& g, float2* S, cudaStream_t st)
{
    const long long n = (long long)g.hw * g.H * nframes;
    import_spectra_kernel<<<grid_for(n, 256), 256, 0, st>>>(reinterpret_cast<const double2*>(spectra), nframes, g.W,
                                                             g.H, g.Hs, g.hw, S);
    note_launches(1);
    return cudaGetLastError();
}

} // namespace smip_gpu
