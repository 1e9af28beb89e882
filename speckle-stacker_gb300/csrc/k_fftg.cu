// k_fftg.cu -- the per-frame transforms for frame sizes that are not powers
// of two (or are larger than the radix-2 kernels' 512): any ncols and nrows
// up to kMaxSide.
//
// The reference builds FFTW plans for whatever size its frames have
// (smip-cli/main.cpp:256-259, crosscorrel.h:112-141), so frames such as
// 100 x 100 or a 320 x 240 crop (-s, main.cpp:157-167) are ordinary input.
// These kernels compute the same quantities as k_fft.cu -- the float-float
// forward transform into the spectrum layout S, the power-spectrum partials,
// the FP32 correlation transforms -- and the FP64 lines of the final image,
// with a mixed-radix transform instead of the radix-2 one.
//
// Transform: the Stockham autosort formulation of the mixed-radix FFT
// (Govindaraju, Lloyd, Dotsenko, Smith, Manferdelli, "High performance
// discrete Fourier transforms on graphics processors", SC 2008).  The length
// L is split into factors R_1 R_2 ... (4 where two 2s pair up, then the
// primes); with Ns the product of the earlier factors, the pass of radix R
// maps x to y by
//     y[(j / Ns) Ns R + q Ns + k] = sum_{r < R} x[j + r L / R] w^(r (k + q Ns) L / (Ns R)),
//     j in [0, L / R), k = j mod Ns, q in [0, R),  w = exp(-2 pi i / L),
// which folds the pass's twiddle and its radix-R DFT into one table lookup
// per term (exponents reduced mod L exactly in integers).  Each output is one
// thread's sum of R terms read from shared memory; results come out in
// natural order.  Arithmetic per the caller's type: float-float (dfc, the
// same error-free two_prod / two_sum steps as the radix-2 forward transform,
// renormalised after every pass), FP32, or FP64.
#include "smip_dev.cuh"

namespace smip_gpu {

// ---------------------------------------------------------------- arithmetic
__device__ __forceinline__ float2 gmac(float2 acc, float2 x, float2 w)
{
    acc.x = fmaf(x.x, w.x, fmaf(-x.y, w.y, acc.x));
    acc.y = fmaf(x.x, w.y, fmaf(x.y, w.x, acc.y));
    return acc;
}
__device__ __forceinline__ double2 gmac(double2 acc, double2 x, double2 w)
{
    acc.x = fma(x.x, w.x, fma(-x.y, w.y, acc.x));
    acc.y = fma(x.x, w.y, fma(x.y, w.x, acc.y));
    return acc;
}
__device__ __forceinline__ dfc gmac(const dfc& acc, const dfc& x, const dfc& w) { return df_cadd(acc, df_cmul(x, w)); }
__device__ __forceinline__ float2 gconj(float2 w) { return make_float2(w.x, -w.y); }
__device__ __forceinline__ double2 gconj(double2 w) { return make_double2(w.x, -w.y); }
__device__ __forceinline__ dfc gconj(dfc w) { return tw_conj(w); }
__device__ __forceinline__ float2 gnorm(float2 v) { return v; }
__device__ __forceinline__ double2 gnorm(double2 v) { return v; }
__device__ __forceinline__ dfc gnorm(dfc v)
{
    df_norm(v.h.x, v.l.x);
    df_norm(v.h.y, v.l.y);
    return v;
}

// Stockham passes over nl lines of length p.L (line stride ls) in shared
// memory, ping-ponging between x and y; returns the buffer with the result.
// tw: p.L entries exp(-2 pi i k / L); sign -1 forward, +1 inverse
// (unnormalised).  Called by all threads of the block.
template <typename C>
__device__ C* stockham(C* x, C* y, const GenPlan& p, int nl, int ls, const C* tw, int sign)
{
    const int L = p.L;
    int Ns = 1;
    for (int f = 0; f < p.nf; ++f) {
        const int R = p.fac[f];
        const int LR = L / R;
        const int step = LR / Ns; // L / (Ns R)
        const unsigned* mp = p.map ? p.map + f * L : nullptr;
        for (int idx = threadIdx.x; idx < nl * L; idx += blockDim.x) {
            const int line = idx / L, o = idx - line * L;
            int j, e0;
            if (mp) { // precomputed for this length: no divisions
                const unsigned m = __ldg(mp + o);
                j = (int)(m & 0xffffu);
                e0 = (int)(m >> 16);
            } else {
                const int k = o % Ns, t = o / Ns;
                const int q = t % R;
                j = (t / R) * Ns + k;
                e0 = (k + q * Ns) * step; // < L
            }
            const C* X = x + line * ls + j;
            C acc = X[0];
            int e = 0;
            for (int r = 1; r < R; ++r) {
                e += e0;
                if (e >= L)
                    e -= L;
                const C w = sign > 0 ? gconj(tw[e]) : tw[e];
                acc = gmac(acc, X[r * LR], w);
            }
            y[line * ls + o] = gnorm(acc);
        }
        __syncthreads();
        C* tmp = x;
        x = y;
        y = tmp;
        Ns *= R;
    }
    return x;
}

template <typename C> __device__ void load_table(C* dst, const C* src, int n)
{
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        dst[k] = src[k];
}

template <typename T> __device__ __forceinline__ dfc pix_dfc(const T* p, long long i)
{
    dfc d;
    d.h = make_float2((float)p[i], 0.f); // u8/u16/f32 are exact in FP32
    d.l = make_float2(0.f, 0.f);
    return d;
}
template <> __device__ __forceinline__ dfc pix_dfc<double>(const double* p, long long i)
{
    const double v = p[i];
    const float h = (float)v;
    dfc d;
    d.h = make_float2(h, 0.f);
    d.l = make_float2((float)(v - (double)h), 0.f);
    return d;
}

__device__ __forceinline__ float2 dfc_round(const dfc& v) { return make_float2(v.h.x + v.l.x, v.h.y + v.l.y); }

// ---------------------------------------------------------------- row pass
// rb rows of one frame per CTA: forward float-float transform of each real
// row; writes G'(a, y) = sum_x f(x, y) exp(+2 pi i a x / W) = X[(W - a) mod W],
// a < hw, stored [f][a][y] (the layout of k_fft.cu's row pass).  copy_out:
// the frames as read, written to device memory (mapped host input).
template <typename T>
__global__ void __launch_bounds__(256) gen_row_kernel(const T* __restrict__ frames, long long fstride, int H, int hw,
                                                      int rb, const GenPlan pw, const dfc* __restrict__ tw_g,
                                                      dfc* __restrict__ Gt, T* __restrict__ copy_out)
{
    extern __shared__ dfc smg[];
    const int W = pw.L;
    dfc* tw = smg;
    dfc* X = tw + W;
    dfc* Y = X + rb * W;
    const int f = blockIdx.y;
    const int y0 = blockIdx.x * rb;
    const int nr = min(rb, H - y0);
    const T* fr = frames + (long long)f * fstride + (long long)y0 * W;
    T* co = copy_out ? copy_out + (long long)f * fstride + (long long)y0 * W : nullptr;
    load_table(tw, tw_g, W);
    for (int i = threadIdx.x; i < nr * W; i += blockDim.x) {
        X[i] = pix_dfc(fr, i);
        if (co)
            co[i] = fr[i];
    }
    __syncthreads();
    const dfc* Z = stockham(X, Y, pw, nr, W, tw, -1);
    dfc* out = Gt + (long long)f * hw * H;
    for (int i = threadIdx.x; i < hw * nr; i += blockDim.x) {
        const int a = i / nr, r = i - a * nr;
        out[(long long)a * H + y0 + r] = Z[r * W + (a == 0 ? 0 : W - a)];
    }
}

// ------------------------------------------------------------- column pass
// One CTA per (a, chunk of frames), cl columns at a time: float-float forward
// transform along y gives F(-a, y); writes S[f][a][c] = F(-a, c - H/2) (row
// pitch Hs, rounded to FP32), the power partials |F|^2 summed in float-float
// in frame order, and the FP32 inverse y-transform of conj(R) * F into T.
// mode 1: frame 0 only, its spectrum F(-a, y) into Rout (y in natural order).
__global__ void __launch_bounds__(256) gen_col_kernel(int mode, const dfc* __restrict__ Gt, float2* __restrict__ S,
                                                      int Hs, const float2* __restrict__ Rbuf, float2* __restrict__ Rout,
                                                      float2* __restrict__ T, double* __restrict__ Ppart, int nframes,
                                                      int fpc, int skip_xcorr_frame0, int hw, int cl, const GenPlan ph,
                                                      const dfc* __restrict__ twd_g, const float2* __restrict__ tw_g)
{
    extern __shared__ dfc smg[];
    const int H = ph.L;
    dfc* twd = smg;                                                // [H]
    dfc* X = twd + H;                                              // [cl][H]
    dfc* Y = X + cl * H;                                           // [cl][H]
    float2* tw = reinterpret_cast<float2*>(Y + cl * H);            // [H]
    float2* R = tw + H;                                            // [H]
    float2* X2 = R + H;                                            // [cl][H]
    float2* Y2 = X2 + cl * H;                                      // [cl][H]
    float2* pacc = Y2 + cl * H;                                    // [H] float-float (hi, lo)
    const int a = blockIdx.x;
    const int chunk = blockIdx.y;
    const int fbeg = chunk * fpc;
    const int fend = min(nframes, fbeg + fpc);
    const long long gstride = (long long)hw * H;
    const long long sstride = (long long)hw * Hs;
    const int hh = H / 2;
    load_table(twd, twd_g, H);
    load_table(tw, tw_g, H);
    if (mode == 0)
        for (int y = threadIdx.x; y < H; y += blockDim.x) {
            R[y] = Rbuf[(long long)a * H + y];
            pacc[y] = make_float2(0.f, 0.f);
        }
    for (int f0 = fbeg; f0 < fend; f0 += cl) {
        const int nl = min(cl, fend - f0);
        __syncthreads();
        for (int i = threadIdx.x; i < nl * H; i += blockDim.x) {
            const int l = i / H, y = i - l * H;
            X[i] = Gt[(f0 + l) * gstride + (long long)a * H + y];
        }
        __syncthreads();
        const dfc* Fm = stockham(X, Y, ph, nl, H, twd, -1); // Fm[l][y] = F(-a, y)
        if (mode == 1) {
            for (int y = threadIdx.x; y < H; y += blockDim.x)
                Rout[(long long)a * H + y] = dfc_round(Fm[y]);
            return;
        }
        for (int i = threadIdx.x; i < nl * H; i += blockDim.x) {
            const int l = i / H, c = i - l * H;
            int y = c - hh;
            y += y < 0 ? H : 0;
            S[(f0 + l) * sstride + (long long)a * Hs + c] = dfc_round(Fm[l * H + y]);
        }
        // power spectrum, frames in order per element, float-float sums
        for (int c = threadIdx.x; c < H; c += blockDim.x) {
            int y = c - hh;
            y += y < 0 ? H : 0;
            float ah = pacc[c].x, al = pacc[c].y;
            for (int l = 0; l < nl; ++l) {
                dfc v = Fm[l * H + y];
                float rh, rl, ih, il, sh, sl;
                df_mul(v.h.x, v.l.x, v.h.x, v.l.x, rh, rl);
                df_mul(v.h.y, v.l.y, v.h.y, v.l.y, ih, il);
                df_add(rh, rl, ih, il, sh, sl);
                df_add(ah, al, sh, sl, ah, al);
            }
            pacc[c] = make_float2(ah, al);
        }
        // correlation product conj(R) * F in FP32, inverse y-transform
        for (int i = threadIdx.x; i < nl * H; i += blockDim.x) {
            const int y = i % H;
            const float2 r = R[y], v = dfc_round(Fm[i]);
            X2[i] = make_float2(r.x * v.x + r.y * v.y, r.x * v.y - r.y * v.x);
        }
        __syncthreads();
        const float2* Tz = stockham(X2, Y2, ph, nl, H, tw, +1);
        for (int i = threadIdx.x; i < nl * H; i += blockDim.x) {
            const int l = i / H, y = i - l * H;
            if (skip_xcorr_frame0 && f0 + l == 0)
                continue;
            T[(f0 + l) * gstride + (long long)a * H + y] = Tz[i];
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < H; c += blockDim.x)
        Ppart[(long long)chunk * gstride + (long long)a * H + c] = (double)pacc[c].x + (double)pacc[c].y;
}

// ------------------------------------------------------- correlation rows
// c2r along x of T(-a, y): Z(0) = Re T(0); Z(k) = conj T(a = k) for
// 0 < k < W/2; Re T(W/2) at the Nyquist column of an even W (FFTW's c2r
// ignores those imaginary parts); Z(k) = T(a = W - k) above.  Output: the
// correlation c[y][x] and each row's maximum.
__global__ void __launch_bounds__(256) gen_xrows_kernel(const float2* __restrict__ Tg, float* __restrict__ corr,
                                                        float* __restrict__ rowmax, int H, int hw, int rb,
                                                        const GenPlan pw, const float2* __restrict__ tw_g)
{
    extern __shared__ float2 smx[];
    const int W = pw.L;
    float2* tw = smx;
    float2* X = tw + W;
    float2* Y = X + rb * W;
    const int f = blockIdx.y;
    const int y0 = blockIdx.x * rb;
    const int nr = min(rb, H - y0);
    const float2* T = Tg + (long long)f * hw * H;
    load_table(tw, tw_g, W);
    for (int i = threadIdx.x; i < nr * W; i += blockDim.x) {
        const int r = i / W, k = i - r * W;
        const int y = y0 + r;
        float2 z;
        if (k == 0)
            z = make_float2(T[y].x, 0.f);
        else if (2 * k == W)
            z = make_float2(T[(long long)k * H + y].x, 0.f);
        else if (2 * k < W)
            z = gconj(T[(long long)k * H + y]);
        else
            z = T[(long long)(W - k) * H + y];
        X[i] = z;
    }
    __syncthreads();
    const float2* Z = stockham(X, Y, pw, nr, W, tw, +1);
    float* out = corr + (long long)f * W * H + (long long)y0 * W;
    for (int i = threadIdx.x; i < nr * W; i += blockDim.x)
        out[i] = Z[i].x;
    // each row's maximum, one warp per row
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < nr; r += blockDim.x >> 5) {
        float m = -INFINITY;
        for (int x = lane; x < W; x += 32)
            m = fmaxf(m, Z[r * W + x].x);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0)
            rowmax[(long long)f * H + y0 + r] = m;
    }
}

// -------------------------------------------------------------- FP64 lines
// nlb lines per CTA of length p.L (element stride es, line stride ls), in place.
__global__ void __launch_bounds__(256) gen_lines_d_kernel(double2* __restrict__ data, int nlines, long long ls,
                                                          long long es, int sign, int nlb, const GenPlan p,
                                                          const double2* __restrict__ tw_g)
{
    extern __shared__ double2 smd2[];
    const int L = p.L;
    double2* tw = smd2;
    double2* X = tw + L;
    double2* Y = X + nlb * L;
    const int l0 = blockIdx.x * nlb;
    const int nl = min(nlb, nlines - l0);
    load_table(tw, tw_g, L);
    for (int i = threadIdx.x; i < nl * L; i += blockDim.x) {
        const int l = i / L, k = i - l * L;
        X[i] = data[(l0 + l) * ls + k * es];
    }
    __syncthreads();
    const double2* Z = stockham(X, Y, p, nl, L, tw, sign);
    for (int i = threadIdx.x; i < nl * L; i += blockDim.x) {
        const int l = i / L, k = i - l * L;
        data[(l0 + l) * ls + k * es] = Z[i];
    }
}

// ------------------------------------------------------------- launchers
// Blocking per launch, chosen so that a CTA's shared memory stays below
// kGenSmem for every length up to kMaxSide.
constexpr size_t kGenSmem = 200 * 1024;
// Lines per CTA: as many as fit in about 64 KB of shared memory, so that
// several CTAs share an SM and hide each other's shared-memory latency
// (one CTA of 200 KB per SM left the schedulers idle more than half the time).
constexpr long kGenTarget = 64 * 1024;

static int row_block(int W) { return (int)std::max(1L, std::min(16L, (kGenTarget / (16L * W) - 1) / 2)); }
static size_t row_smem(int W, int rb) { return sizeof(dfc) * (size_t)W * (1 + 2 * rb); }
static int col_lines(int H)
{
    const long per = (long)H * (2 * sizeof(dfc) + 2 * sizeof(float2)); // one more column
    const long fixed = (long)H * (sizeof(dfc) + 3 * sizeof(float2));
    return (int)std::max(1L, std::min(8L, (kGenTarget - fixed) / per));
}
static size_t col_smem(int H, int cl)
{
    return (size_t)H * (sizeof(dfc) * (1 + 2 * cl) + sizeof(float2) * (3 + 2 * cl));
}
static int xrow_block(int W) { return (int)std::max(1L, std::min(16L, (kGenTarget / (8L * W) - 1) / 2)); }
static size_t xrow_smem(int W, int rb) { return sizeof(float2) * (size_t)W * (1 + 2 * rb); }
static int lines_block(int L) { return (int)std::max(1L, std::min(8L, (kGenTarget / (16L * L) - 1) / 2)); }
static size_t lines_smem(int L, int nlb) { return sizeof(double2) * (size_t)L * (1 + 2 * nlb); }

template <typename K> static cudaError_t allow(K kern, size_t bytes)
{
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

size_t gen_max_smem() { return kGenSmem; }

cudaError_t launch_gen_row_pass(int dtype, const void* frames, long long fstride, int nframes, const Geometry& g,
                                dfc* Gt, const dfc* twW, cudaStream_t st, void* copy_out)
{
    const int rb = row_block(g.W);
    const dim3 grid((g.H + rb - 1) / rb, nframes);
    const size_t smem = row_smem(g.W, rb);
    cudaError_t e = cudaSuccess;
#define SMIP_GEN_ROW(TY)                                                                                          \
    if ((e = allow(gen_row_kernel<TY>, kGenSmem)) != cudaSuccess)                                                 \
        return e;                                                                                                  \
    gen_row_kernel<TY><<<grid, 256, smem, st>>>((const TY*)frames, fstride, g.H, g.hw, rb, g.pW, twW, Gt,         \
                                                (TY*)copy_out);
    switch (dtype) {
    case 0: SMIP_GEN_ROW(uint8_t) break;
    case 1: SMIP_GEN_ROW(uint16_t) break;
    case 2: SMIP_GEN_ROW(float) break;
    default: SMIP_GEN_ROW(double) break;
    }
#undef SMIP_GEN_ROW
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_gen_col_pass(int mode, const dfc* Gt, float2* S, const float2* Rbuf, float2* Rout, float2* T,
                                double* Ppart, int nframes, int fpc, int skip_xcorr_frame0, const Geometry& g,
                                const dfc* twH, const float2* twH32, cudaStream_t st)
{
    const int nchunks = mode == 1 ? 1 : (nframes + fpc - 1) / fpc;
    const int cl = col_lines(g.H);
    const dim3 grid(g.hw, nchunks);
    cudaError_t e = allow(gen_col_kernel, kGenSmem);
    if (e != cudaSuccess)
        return e;
    gen_col_kernel<<<grid, 256, col_smem(g.H, cl), st>>>(mode, Gt, S, g.Hs, Rbuf, Rout, T, Ppart,
                                                         mode == 1 ? 1 : nframes, fpc, skip_xcorr_frame0, g.hw, cl,
                                                         g.pH, twH, twH32);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_gen_xcorr_rows(const float2* T, float* corr, float* rowmax, int nframes, const Geometry& g,
                                  const float2* twW32, cudaStream_t st)
{
    const int rb = xrow_block(g.W);
    const dim3 grid((g.H + rb - 1) / rb, nframes);
    cudaError_t e = allow(gen_xrows_kernel, kGenSmem);
    if (e != cudaSuccess)
        return e;
    gen_xrows_kernel<<<grid, 256, xrow_smem(g.W, rb), st>>>(T, corr, rowmax, g.H, g.hw, rb, g.pW, twW32);
    note_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_gen_lines_d(double2* data, const GenPlan& p, int nlines, long long ls, long long es, int sign,
                               const double2* tw, cudaStream_t st)
{
    const int nlb = lines_block(p.L);
    cudaError_t e = allow(gen_lines_d_kernel, kGenSmem);
    if (e != cudaSuccess)
        return e;
    gen_lines_d_kernel<<<(nlines + nlb - 1) / nlb, 256, lines_smem(p.L, nlb), st>>>(data, nlines, ls, es, sign, nlb,
                                                                                    p, tw);
    note_launches(1);
    return cudaGetLastError();
}

// Factors of L for the Stockham passes: pairs of 2 as 4, a remaining 2, then
// the odd primes in increasing order.
GenPlan make_gen_plan(int L)
{
    GenPlan p {};
    p.L = L;
    int n = L, twos = 0;
    while (n % 2 == 0) {
        n /= 2;
        ++twos;
    }
    for (; twos >= 2; twos -= 2)
        p.fac[p.nf++] = 4;
    if (twos)
        p.fac[p.nf++] = 2;
    for (int q = 3; q <= n; q += 2)
        while (n % q == 0) {
            p.fac[p.nf++] = q;
            n /= q;
        }
    return p;
}

} // namespace smip_gpu
