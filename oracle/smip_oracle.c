/*
 * smip_oracle.c -- CPU oracle for the SMIP hot path (TEST INFRASTRUCTURE).
 *
 * Plain-C restatement of hangeza/speckle-stacker v0.3.2, one function per
 * reference routine, each citing the reference file:line it follows.  It is
 * the checker for the CUDA library and the CPU baseline of the benchmark; the
 * product path never calls it.
 *
 * Build flags matter: this file is compiled with -ffp-contract=off and without
 * -ffast-math so that every float/double operation rounds exactly as written
 * (no FMA contraction on aarch64, no reassociation), which makes its results
 * identical on x86_64 and aarch64 and bit-identical to the reference headers
 * compiled without fast-math (oracle/ref/).
 */
#include "smip_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793238462643383279502884
#define ORC_2PI (2.0 * ORC_PI)
#define ORC_DBL_EPS 2.220446049250313080847263336181640625e-16 /* constants.h:20 */

/* ------------------------------------------------------------------------ */
/* bispectrum descriptor: include/bispectrum.h:143-160, 203-220              */
/* ------------------------------------------------------------------------ */
void orc_bispec_describe(long ncols, long nrows, long d2, long d3, orc_bispec_desc* d)
{
    long dims[4] = { ncols, nrows, d2, d3 };
    memset(d, 0, sizeof(*d));
    d->base_size = 1;
    d->totalsize = 1;
    for (int n = 0; n < 4; ++n) {
        d->dimsizes[n] = dims[n];
        d->sizes[n] = (dims[n] / 2) * 2 + 1;                          /* :207-210 */
        d->base_sizes[n] = (n == 0 || n == 2) ? d->sizes[n] - d->sizes[n] / 2 : d->sizes[n]; /* :217-219 */
        d->base_size *= d->base_sizes[n];
        d->totalsize *= d->sizes[n];
        d->min_idx[n] = -(int)d->sizes[n] / 2;                        /* :151-153 */
        d->max_idx[n] = (int)d->sizes[n] + d->min_idx[n] - 1;         /* :154-158 */
    }
}

/* include/bispectrum.h:324-349.  Arithmetic is done modulo 2^64 exactly as the
 * reference's size_t arithmetic, so out-of-range indices alias silently. */
static uint64_t calc_offset_u64(const orc_bispec_desc* d, const int idx_in[4])
{
    int idx[4] = { -idx_in[0], idx_in[1], -idx_in[2], idx_in[3] };
    for (int n = 0; n < 4; ++n) {
        if (idx[n] < 0)
            idx[n] = (int)((uint64_t)(int64_t)idx[n] + (uint64_t)d->sizes[n]);
    }
    uint64_t addr = (uint64_t)(int64_t)idx[0];
    addr *= (uint64_t)d->base_sizes[1];
    addr += (uint64_t)(int64_t)idx[1];
    addr *= (uint64_t)d->base_sizes[2];
    addr += (uint64_t)(int64_t)idx[2];
    addr *= (uint64_t)d->base_sizes[3];
    addr += (uint64_t)(int64_t)idx[3];
    return addr;
}

long orc_calc_offset(const orc_bispec_desc* d, const int idx[4])
{
    return (long)calc_offset_u64(d, idx);
}

/* include/bispectrum.h:280-316 */
void orc_calc_indices(const orc_bispec_desc* d, long addr, int idx[4])
{
    long temp = d->base_size / d->base_sizes[0];
    long rest = addr;
    long a0 = rest / temp;
    rest -= temp * a0;
    temp = d->base_sizes[2] * d->base_sizes[3];
    long a1 = rest / temp;
    rest -= temp * a1;
    temp = d->base_sizes[3];
    long a2 = rest / temp;
    rest -= temp * a2;
    long a[4] = { a0, a1, a2, rest };
    for (int n = 0; n < 4; ++n) {
        int v = (int)a[n];
        idx[n] = v > (int)d->sizes[n] / 2 ? (int)(v - d->sizes[n]) : v;
    }
    idx[0] = -idx[0];
    idx[2] = -idx[2];
}

/* include/bispectrum.h:162-174 (classify) and 553-589 (canonicalize) */
static void canonicalize(const int in[4], int out[4], int* conj)
{
    const int i0 = in[0], i1 = in[1], i2 = in[2], i3 = in[3];
    *conj = 0;
    if (i0 <= 0 && i2 <= 0) { /* T1 */
        out[0] = i0; out[1] = i1; out[2] = i2; out[3] = i3;
    } else if (i0 > 0 && i2 > 0) { /* T7 */
        *conj = 1;
        out[0] = -i0; out[1] = -i1; out[2] = -i2; out[3] = -i3;
    } else if (i0 > 0 && i2 <= 0) {
        if (i0 + i2 > 0) { /* T6 */
            out[0] = -i0 - i2; out[1] = -i1 - i3; out[2] = i2; out[3] = i3;
        } else { /* T9 */
            *conj = 1;
            out[0] = -i0; out[1] = -i1; out[2] = i2 + i0; out[3] = i3 + i1;
        }
    } else { /* i0 <= 0 && i2 > 0 */
        if (i0 + i2 > 0) { /* T3 */
            out[0] = i0; out[1] = i1; out[2] = -i2 - i0; out[3] = -i3 - i1;
        } else { /* T12 */
            *conj = 1;
            out[0] = i0 + i2; out[1] = i1 + i3; out[2] = -i2; out[3] = -i3;
        }
    }
}

/* include/bispectrum.h:482-512 */
long orc_get_element_offset(const orc_bispec_desc* d, const int idx_in[4], int* conj)
{
    int idx[4] = { idx_in[0], idx_in[1], idx_in[2], idx_in[3] };
    const int* mx = d->max_idx;
    if (abs(idx[2]) > mx[2] || abs(idx[3]) > mx[3]) {               /* :487-490 */
        int t = idx[0]; idx[0] = idx[2]; idx[2] = t;
        t = idx[1]; idx[1] = idx[3]; idx[3] = t;
    }
    for (int n = 0; n < 4; ++n)                                       /* :491-493 */
        if (idx[n] < d->min_idx[n] || idx[n] > mx[n])
            return -1;
    int uv[4];
    canonicalize(idx, uv, conj);                                      /* :495-496 */
    if (abs(uv[2]) > mx[2] || abs(uv[3]) > mx[3]) {                 /* :498-501 */
        int t = uv[0]; uv[0] = uv[2]; uv[2] = t;
        t = uv[1]; uv[1] = uv[3]; uv[3] = t;
    }
    uint64_t addr = calc_offset_u64(d, uv);                           /* :503 */
    if (addr >= (uint64_t)d->base_size)                               /* :505-507 */
        return -1;
    return (long)addr;
}

/* ------------------------------------------------------------------------ */
/* FFT: stand-in for the FFTW3 calls of smip-cli/main.cpp:256-259, 340-346  */
/* and include/crosscorrel.h:112-141.  Unnormalised, FFTW sign convention.  */
/* Radix-2 for powers of two, direct DFT otherwise.                          */
/* ------------------------------------------------------------------------ */
typedef struct {
    long n;
    int sign;
    double* tw; /* n complex: exp(sign*2*pi*i*k/n) */
} orc_plan;

static void plan_init(orc_plan* p, long n, int sign)
{
    p->n = n;
    p->sign = sign;
    p->tw = (double*)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    for (long k = 0; k < n; ++k) {
        double a = ORC_2PI * (double)k / (double)n;
        p->tw[2 * k] = cos(a);
        p->tw[2 * k + 1] = (double)sign * sin(a);
    }
}

static void plan_free(orc_plan* p) { free(p->tw); }

static int is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }

/* in-place 1-D transform of n complex values (contiguous); work: n complex */
static void fft_1d(const orc_plan* p, double* x, double* work)
{
    const long n = p->n;
    if (n <= 1)
        return;
    if (is_pow2(n)) {
        /* bit reversal */
        for (long i = 1, j = 0; i < n; ++i) {
            long bit = n >> 1;
            for (; j & bit; bit >>= 1)
                j ^= bit;
            j ^= bit;
            if (i < j) {
                double tr = x[2 * i], ti = x[2 * i + 1];
                x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
                x[2 * j] = tr; x[2 * j + 1] = ti;
            }
        }
        for (long len = 2; len <= n; len <<= 1) {
            const long half = len >> 1;
            const long step = n / len;
            for (long s = 0; s < n; s += len) {
                for (long k = 0; k < half; ++k) {
                    const double wr = p->tw[2 * (k * step)], wi = p->tw[2 * (k * step) + 1];
                    double* a = x + 2 * (s + k);
                    double* b = x + 2 * (s + k + half);
                    const double br = b[0] * wr - b[1] * wi;
                    const double bi = b[0] * wi + b[1] * wr;
                    b[0] = a[0] - br; b[1] = a[1] - bi;
                    a[0] = a[0] + br; a[1] = a[1] + bi;
                }
            }
        }
    } else {
        for (long k = 0; k < n; ++k) {
            double sr = 0.0, si = 0.0;
            for (long j = 0; j < n; ++j) {
                const long m = (j * k) % n;
                const double wr = p->tw[2 * m], wi = p->tw[2 * m + 1];
                sr += x[2 * j] * wr - x[2 * j + 1] * wi;
                si += x[2 * j] * wi + x[2 * j + 1] * wr;
            }
            work[2 * k] = sr;
            work[2 * k + 1] = si;
        }
        memcpy(x, work, sizeof(double) * 2 * (size_t)n);
    }
}

void orc_fft_2d(double* data, long nrows, long ncols, int sign)
{
    orc_plan pr, pc;
    plan_init(&pr, ncols, sign);
    plan_init(&pc, nrows, sign);
    long m = ncols > nrows ? ncols : nrows;
    double* work = (double*)malloc(sizeof(double) * 2 * (size_t)m);
    double* col = (double*)malloc(sizeof(double) * 2 * (size_t)m);
    for (long y = 0; y < nrows; ++y)
        fft_1d(&pr, data + 2 * y * ncols, work);
    for (long x = 0; x < ncols; ++x) {
        for (long y = 0; y < nrows; ++y) {
            col[2 * y] = data[2 * (x + y * ncols)];
            col[2 * y + 1] = data[2 * (x + y * ncols) + 1];
        }
        fft_1d(&pc, col, work);
        for (long y = 0; y < nrows; ++y) {
            data[2 * (x + y * ncols)] = col[2 * y];
            data[2 * (x + y * ncols) + 1] = col[2 * y + 1];
        }
    }
    free(work);
    free(col);
    plan_free(&pr);
    plan_free(&pc);
}

void orc_fft_r2c_2d(const double* in, double* out, long nrows, long ncols)
{
    const long hc = ncols / 2 + 1;
    double* full = (double*)malloc(sizeof(double) * 2 * (size_t)(nrows * ncols));
    for (long i = 0; i < nrows * ncols; ++i) {
        full[2 * i] = in[i];
        full[2 * i + 1] = 0.0;
    }
    orc_fft_2d(full, nrows, ncols, -1);
    for (long y = 0; y < nrows; ++y)
        for (long x = 0; x < hc; ++x) {
            out[2 * (x + y * hc)] = full[2 * (x + y * ncols)];
            out[2 * (x + y * hc) + 1] = full[2 * (x + y * ncols) + 1];
        }
    free(full);
}

void orc_fft_c2r_2d(const double* in, double* out, long nrows, long ncols)
{
    const long hc = ncols / 2 + 1;
    double* full = (double*)malloc(sizeof(double) * 2 * (size_t)(nrows * ncols));
    for (long y = 0; y < nrows; ++y) {
        for (long x = 0; x < ncols; ++x) {
            double re, im;
            if (x < hc) {
                re = in[2 * (x + y * hc)];
                im = in[2 * (x + y * hc) + 1];
            } else {
                const long yy = (nrows - y) % nrows;
                const long xx = ncols - x;
                re = in[2 * (xx + yy * hc)];
                im = -in[2 * (xx + yy * hc) + 1];
            }
            full[2 * (x + y * ncols)] = re;
            full[2 * (x + y * ncols) + 1] = im;
        }
    }
    orc_fft_2d(full, nrows, ncols, +1);
    for (long i = 0; i < nrows * ncols; ++i)
        out[i] = full[2 * i];
    free(full);
}

/* ------------------------------------------------------------------------ */
/* bispectrum accumulation: include/bispectrum.h:356-409                     */
/* ------------------------------------------------------------------------ */
typedef struct {
    float* b32;
    double* b64;
    const float* f32;  /* narrowed spectrum (bispectrum.h:399 T t{...}) */
    const double* f64;
    const orc_bispec_desc* d;
    long ncols, nrows;
    int min1, min2, min3, min4, max1, max2, max4;
    int i_lo, i_hi; /* this worker's slice of the u_x loop */
} acc_job;

static inline long wrap_at(int x, int y, long ncols, long nrows)
{
    /* Array2::at, include/array2.h:327-339 */
    long xx = x < 0 ? x + ncols : x;
    long yy = y < 0 ? y + nrows : y;
    return xx + yy * ncols;
}

static void* acc_worker(void* arg)
{
    const acc_job* J = (const acc_job*)arg;
    const long nc = J->ncols, nr = J->nrows;
    for (int i = J->i_lo; i <= J->i_hi; i++) {
        for (int j = J->min2; j <= J->max2; j++) {
            for (int k = J->min3; k <= 0; k++) {
                for (int l = J->min4; l <= J->max4; l++) {
                    if (((i + k) >= J->min1) && ((j + l) >= J->min2)
                        && ((i + k) <= J->max1) && ((j + l) <= J->max2)) {
                        const long pu = wrap_at(i, j, nc, nr);
                        const long pv = wrap_at(k, l, nc, nr);
                        const long pw = wrap_at(i + k, j + l, nc, nr);
                        const int idx[4] = { i, j, k, l };
                        const uint64_t off = calc_offset_u64(J->d, idx);
                        if (J->b32) {
                            /* complex<float>: t = F(u); t *= F(v); t *= conj F(u+v) */
                            const float ar = J->f32[2 * pu], ai = J->f32[2 * pu + 1];
                            const float br = J->f32[2 * pv], bi = J->f32[2 * pv + 1];
                            const float cr = J->f32[2 * pw], ci = -J->f32[2 * pw + 1];
                            const float tr = ar * br - ai * bi;
                            const float ti = ar * bi + ai * br;
                            const float sr = tr * cr - ti * ci;
                            const float si = tr * ci + ti * cr;
                            J->b32[2 * off] += sr;
                            J->b32[2 * off + 1] += si;
                        } else {
                            const double ar = J->f64[2 * pu], ai = J->f64[2 * pu + 1];
                            const double br = J->f64[2 * pv], bi = J->f64[2 * pv + 1];
                            const double cr = J->f64[2 * pw], ci = -J->f64[2 * pw + 1];
                            const double tr = ar * br - ai * bi;
                            const double ti = ar * bi + ai * br;
                            const double sr = tr * cr - ti * ci;
                            const double si = tr * ci + ti * cr;
                            J->b64[2 * off] += sr;
                            J->b64[2 * off + 1] += si;
                        }
                    }
                }
            }
        }
    }
    return NULL;
}

static void accumulate_common(float* b32, double* b64, const double* fft, long ncols, long nrows,
                              long depth, int nthreads)
{
    orc_bispec_desc d;
    orc_bispec_describe(ncols, nrows, depth, depth, &d);
    /* Array2::min_sindices / max_sindices, include/array2.h:675-688 */
    const int fmin0 = -(int)(ncols >> 1), fmin1 = -(int)(nrows >> 1);
    const int fmax0 = -(int)ncols / 2 + (int)ncols - 1, fmax1 = -(int)nrows / 2 + (int)nrows - 1;
    acc_job base;
    memset(&base, 0, sizeof(base));
    base.b32 = b32;
    base.b64 = b64;
    base.d = &d;
    base.ncols = ncols;
    base.nrows = nrows;
    /* bispectrum.h:383-391 */
    base.min1 = fmin0 > d.min_idx[0] ? fmin0 : d.min_idx[0];
    base.min2 = fmin1 > d.min_idx[1] ? fmin1 : d.min_idx[1];
    base.min3 = fmin0 > d.min_idx[2] ? fmin0 : d.min_idx[2];
    base.min4 = fmin1 > d.min_idx[3] ? fmin1 : d.min_idx[3];
    base.max1 = fmax0 < d.max_idx[0] ? fmax0 : d.max_idx[0];
    base.max2 = fmax1 < d.max_idx[1] ? fmax1 : d.max_idx[1];
    base.max4 = fmax1 < d.max_idx[3] ? fmax1 : d.max_idx[3];
    float* f32 = NULL;
    if (b32) {
        f32 = (float*)malloc(sizeof(float) * 2 * (size_t)(ncols * nrows));
        for (long n = 0; n < 2 * ncols * nrows; ++n)
            f32[n] = (float)fft[n];
        base.f32 = f32;
    } else {
        base.f64 = fft;
    }
    const int ni = base.min1 <= 0 ? 1 - base.min1 : 0;
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > ni)
        nthreads = ni > 0 ? ni : 1;
    if (nthreads == 1) {
        base.i_lo = base.min1;
        base.i_hi = 0;
        acc_worker(&base);
    } else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        acc_job* jobs = (acc_job*)malloc(sizeof(acc_job) * (size_t)nthreads);
        for (int t = 0; t < nthreads; ++t) {
            jobs[t] = base;
            jobs[t].i_lo = base.min1 + (int)((long)ni * t / nthreads);
            jobs[t].i_hi = base.min1 + (int)((long)ni * (t + 1) / nthreads) - 1;
            pthread_create(&th[t], NULL, acc_worker, &jobs[t]);
        }
        for (int t = 0; t < nthreads; ++t)
            pthread_join(th[t], NULL);
        free(th);
        free(jobs);
    }
    free(f32);
}

void orc_accumulate_f32(float* B, const double* fft, long ncols, long nrows, long depth, int nthreads)
{
    accumulate_common(B, NULL, fft, ncols, nrows, depth, nthreads);
}

void orc_accumulate_f64(double* B, const double* fft, long ncols, long nrows, long depth, int nthreads)
{
    accumulate_common(NULL, B, fft, ncols, nrows, depth, nthreads);
}

/* ------------------------------------------------------------------------ */
/* closure-phase recovery                                                    */
/* ------------------------------------------------------------------------ */
/* src/phasereco.cpp:17-36 */
void orc_next_reco_index(double* r, double* phi, int* i, int* j)
{
    const double dr = 1.0;
    const double dphi = 1.0 / (ORC_2PI * *r);
    int ii = *i;
    int jj = *j;
    while ((*i == ii) && (*j == jj)) {
        if ((*phi += dphi) > ORC_2PI) {
            *phi = 0;
            *r += dr;
        }
        ii = (int)(*r * cos(*phi));
        jj = (int)(*r * sin(*phi));
    }
    *i = ii;
    *j = jj;
}

/* include/phasereco.h:56-68: the visit sequence of the reconstruction loop */
long orc_reco_visits(double reco_radius, int* out_ij, long cap)
{
    double r = 0.0, phi = 0.0;
    int i = 0, j = 0;
    long n = 0;
    while (r <= reco_radius) {
        orc_next_reco_index(&r, &phi, &i, &j);
        if (out_ij && n < cap) {
            out_ij[2 * n] = i;
            out_ij[2 * n + 1] = j;
        }
        ++n;
    }
    return n;
}

typedef struct {
    const float* b32;
    const double* b64;
    orc_bispec_desc d;
    long xs, ys;
    double* ph;           /* complex<double> xs*ys */
    unsigned char* flag;
    double* cons;
} reco_ctx;

static inline long pm_at(const reco_ctx* c, int x, int y) { return wrap_at(x, y, c->xs, c->ys); }

/* include/phasereco.h:75-123.  Returns -1 where get_element would throw. */
static int calc_phase(reco_ctx* c, int wx, int wy)
{
    const orc_bispec_desc* d = &c->d;
    /* :81-86 */
    if (abs(wx) + abs(wy) <= 1)
        return 0;
    if (wx < d->min_idx[0] || wx > d->max_idx[0] || wy < d->min_idx[1] || wy > d->max_idx[1])
        return 0;
    /* pm.range(): include/array2.h:675-694 */
    const int pmin0 = -(int)(c->xs >> 1), pmin1 = -(int)(c->ys >> 1);
    const int pmax0 = -(int)c->xs / 2 + (int)c->xs - 1, pmax1 = -(int)c->ys / 2 + (int)c->ys - 1;
    /* Only u with v = w-u inside the v range contribute; visiting them in the
     * reference's order (x fastest, then y; range.h:157-192) keeps the
     * phasor sum bit-identical. */
    int ylo = wy - d->max_idx[3], yhi = wy - d->min_idx[3];
    int xlo = wx - d->max_idx[2], xhi = wx - d->min_idx[2];
    if (ylo < pmin1) ylo = pmin1;
    if (yhi > pmax1) yhi = pmax1;
    if (xlo < pmin0) xlo = pmin0;
    if (xhi > pmax0) xhi = pmax0;
    double sr = 0.0, si = 0.0;
    long cnt = 0;
    for (int uy = ylo; uy <= yhi; ++uy) {
        for (int ux = xlo; ux <= xhi; ++ux) {
            const int vx = wx - ux, vy = wy - uy;
            if (vx < d->min_idx[2] || vx > d->max_idx[2] || vy < d->min_idx[3] || vy > d->max_idx[3])
                continue;
            const long pu = pm_at(c, ux, uy), pv = pm_at(c, vx, vy);
            if (!c->flag[pu] || !c->flag[pv])
                continue;
            const int idx[4] = { ux, uy, vx, vy };
            int cj = 0;
            const long off = orc_get_element_offset(d, idx, &cj);
            if (off < 0)
                return -1;
            double tr, ti;
            if (c->b32) {
                tr = (double)c->b32[2 * off];
                ti = (double)c->b32[2 * off + 1];
            } else {
                tr = c->b64[2 * off];
                ti = c->b64[2 * off + 1];
            }
            if (cj)
                ti = -ti;
            /* ph = phases(u) * phases(v) */
            const double ar = c->ph[2 * pu], ai = c->ph[2 * pu + 1];
            const double br = c->ph[2 * pv], bi = c->ph[2 * pv + 1];
            double pr = ar * br - ai * bi;
            double pi = ar * bi + ai * br;
            const double at = hypot(tr, ti);
            if (at > ORC_DBL_EPS) {
                const double at2 = hypot(tr, ti);
                tr = tr / at2;
                ti = ti / at2;
                ti = -ti; /* conj */
                const double qr = pr * tr - pi * ti;
                const double qi = pr * ti + pi * tr;
                const double aq = hypot(qr, qi);
                sr = sr + qr / aq;
                si = si + qi / aq;
                ++cnt;
            }
        }
    }
    if (cnt > 0) {
        const long pw = pm_at(c, wx, wy);
        c->flag[pw] = 1;
        const double mr = sr / (double)cnt, mi = si / (double)cnt;
        const double ab = hypot(mr, mi);
        if (c->cons)
            c->cons[pw] = ab;
        if (ab > ORC_DBL_EPS) {
            c->ph[2 * pw] = mr / ab;
            c->ph[2 * pw + 1] = mi / ab;
        } else {
            c->ph[2 * pw] = 0.0;
            c->ph[2 * pw + 1] = 0.0;
        }
    }
    return 0;
}

/* include/phasereco.h:33-73 */
int orc_reconstruct_phases(const float* bf32, const double* bf64,
                           long xsize, long ysize, long depth, double reco_radius,
                           double* phases, unsigned char* flags, double* consistency)
{
    reco_ctx c;
    c.b32 = bf32;
    c.b64 = bf64;
    orc_bispec_describe(xsize, ysize, depth, depth, &c.d);
    c.xs = xsize;
    c.ys = ysize;
    c.ph = phases;
    c.flag = flags;
    c.cons = consistency;
    memset(phases, 0, sizeof(double) * 2 * (size_t)(xsize * ysize));
    memset(flags, 0, (size_t)(xsize * ysize));
    if (consistency)
        memset(consistency, 0, sizeof(double) * (size_t)(xsize * ysize));
    /* seeds :42-54; conj(1+0i) has a negative-zero imaginary part */
    const int seeds[5][2] = { { 0, 0 }, { 1, 0 }, { 0, 1 }, { -1, 0 }, { 0, -1 } };
    for (int s = 0; s < 5; ++s) {
        const long p = pm_at(&c, seeds[s][0], seeds[s][1]);
        phases[2 * p] = 1.0;
        phases[2 * p + 1] = s < 3 ? 0.0 : -0.0;
        flags[p] = 1;
        if (consistency)
            consistency[p] = 1.0;
    }
    const int pmin0 = -(int)(xsize >> 1), pmin1 = -(int)(ysize >> 1);
    const int pmax0 = -(int)xsize / 2 + (int)xsize - 1, pmax1 = -(int)ysize / 2 + (int)ysize - 1;
    double r = 0.0, phi = 0.0;
    int i = 0, j = 0;
    while (r <= reco_radius) {
        orc_next_reco_index(&r, &phi, &i, &j);
        if (i >= pmin0 && i <= pmax0 && j >= pmin1 && j <= pmax1) {
            if (!flags[pm_at(&c, i, j)]) {
                if (calc_phase(&c, i, j) < 0)
                    return -1;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* cross correlation: include/crosscorrel.h:96-179                           */
/* ------------------------------------------------------------------------ */
void orc_xcorr_displacement(const double* ref, const double* frame, long ncols, long nrows,
                            int* dx, int* dy, double* corr_out)
{
    const long hc = ncols / 2 + 1;
    double* f1 = (double*)malloc(sizeof(double) * 2 * (size_t)(hc * nrows));
    double* f2 = (double*)malloc(sizeof(double) * 2 * (size_t)(hc * nrows));
    double* corr = corr_out ? corr_out : (double*)malloc(sizeof(double) * (size_t)(ncols * nrows));
    orc_fft_r2c_2d(ref, f1, nrows, ncols);                           /* :112-122 */
    orc_fft_r2c_2d(frame, f2, nrows, ncols);
    for (long n = 0; n < hc * nrows; ++n) {                           /* :127-130 */
        const double ar = f1[2 * n], ai = -f1[2 * n + 1];
        const double br = f2[2 * n], bi = f2[2 * n + 1];
        f1[2 * n] = ar * br - ai * bi;
        f1[2 * n + 1] = ar * bi + ai * br;
    }
    orc_fft_c2r_2d(f1, corr, nrows, ncols);                           /* :135-141 */
    /* :171 std::max_element -> first maximum in row-major order */
    long best = 0;
    for (long n = 1; n < ncols * nrows; ++n)
        if (corr[best] < corr[n])
            best = n;
    int sx = (int)(best % ncols), sy = (int)(best / ncols);           /* :172-174 */
    sx -= (sx < (int)(ncols + 1) / 2) ? 0 : (int)ncols;               /* :175-176 */
    sy -= (sy < (int)(nrows + 1) / 2) ? 0 : (int)nrows;
    *dx = sx;
    *dy = sy;
    free(f1);
    free(f2);
    if (!corr_out)
        free(corr);
}

/* include/array2.h:603-622 */
void orc_shifted(const double* in, double* out, long ncols, long nrows, int dx, int dy)
{
    memset(out, 0, sizeof(double) * (size_t)(ncols * nrows));
    const int W = (int)ncols, H = (int)nrows;
#define ORC_CLAMP(v, lo, hi) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
    const int sx = ORC_CLAMP(dx, 0, W - 1), sy = ORC_CLAMP(dy, 0, H - 1);
    const int ex = ORC_CLAMP(dx + W, 1, W), ey = ORC_CLAMP(dy + H, 1, H);
#undef ORC_CLAMP
    for (int row = sy; row < ey; ++row)
        for (int col = sx; col < ex; ++col)
            out[col + (long)row * W] = in[(col - dx) + (long)(row - dy) * W];
}

/* include/window_function.h:70-85 (Hann: alpha = 0.5, :39-46) */
void orc_general_hamming(double* out, long xsize, long ysize, double aperture, double alpha)
{
    const double trigarg = ORC_2PI / aperture;
    const double c1 = alpha, c2 = 1. - alpha;
    const int xmin = -(int)(xsize >> 1), ymin = -(int)(ysize >> 1);
    const int xmax = -(int)xsize / 2 + (int)xsize - 1, ymax = -(int)ysize / 2 + (int)ysize - 1;
    for (int i = xmin; i <= xmax; ++i)
        for (int j = ymin; j <= ymax; ++j) {
            const double t1 = c1 + c2 * cos(trigarg * (double)i);
            const double t2 = c1 + c2 * cos(trigarg * (double)j);
            out[wrap_at(i, j, xsize, ysize)] = t1 * t2;
        }
}

/* ------------------------------------------------------------------------ */
/* output mapping: include/videoio.h:100-156, 178-206                        */
/* ------------------------------------------------------------------------ */
void orc_map_to_color_u16(const double* v, long n, uint16_t* rgb)
{
    const double M = 65535.0; /* std::numeric_limits<uint16_t>::max() */
    for (long q = 0; q < n; ++q) {
        double x = v[q];
        x = isnan(x) ? 0.0 : (x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x)); /* std::clamp(value, 0., 1.) */
        double r, g, b;
        if (x < 0.25) { /* blue rises */
            r = 0.0; g = 0.0; b = M * (4.0 * x);
        } else if (x < 0.5) { /* green rises, blue falls */
            r = 0.0; g = M * (4.0 * x - 1.0); b = M * (2.0 - 4.0 * x);
        } else if (x < 0.75) { /* red rises, green falls */
            r = M * (4.0 * x - 2.0); g = M * (3.0 - 4.0 * x); b = 0.0;
        } else { /* red full, blue rises again */
            r = M; g = 0.0; b = M * (4.0 * x - 3.0);
        }
        /* static_cast<uint16_t>: truncation toward zero */
        rgb[3 * q] = (uint16_t)r;
        rgb[3 * q + 1] = (uint16_t)g;
        rgb[3 * q + 2] = (uint16_t)b;
    }
}

void orc_array2mat_order(const double* in, double* out, long ncols, long nrows, int signed_symmetry)
{
    const long minx = -(ncols / 2), miny = -(nrows / 2); /* Array2::min_sindices */
    for (long i = 0; i < nrows; ++i)
        for (long j = 0; j < ncols; ++j) {
            long sx = j, sy = i;
            if (signed_symmetry) { /* arr.at({jj, ii}), negative indices wrapped by +size */
                sx = j + minx;
                sy = i + miny;
                sx = sx < 0 ? sx + ncols : sx;
                sy = sy < 0 ? sy + nrows : sy;
            }
            out[i * ncols + j] = in[sy * ncols + sx];
        }
}

/* ------------------------------------------------------------------------ */
/* pipeline: smip-cli/main.cpp:246-378                                       */
/* ------------------------------------------------------------------------ */
static double pixel(const void* frames, int dtype, long n)
{
    switch (dtype) {
    case 0: return (double)((const uint8_t*)frames)[n];
    case 1: return (double)((const uint16_t*)frames)[n];
    case 2: return (double)((const float*)frames)[n];
    default: return ((const double*)frames)[n];
    }
}

/* std::norm of complex<double> as libstdc++ computes it: x*x + y*y */
static inline double cnorm(double re, double im)
{
    return re * re + im * im;
}

int orc_accumulate_frames(const void* frames, int dtype, long nframes, long ncols, long nrows,
                          long depth, int nthreads, const double* ref_frame,
                          float* bispec32, double* powerspec_acc, double* sum_acc, int* shifts)
{
    const long np = ncols * nrows;
    double* indata = (double*)malloc(sizeof(double) * 2 * (size_t)np);
    double* absf = (double*)malloc(sizeof(double) * (size_t)np);
    double* shf = (double*)malloc(sizeof(double) * (size_t)np);
    for (long f = 0; f < nframes; ++f) {
        for (long n = 0; n < np; ++n) {
            const double v = pixel(frames, dtype, f * np + n);
            indata[2 * n] = v;
            indata[2 * n + 1] = 0.0;
            absf[n] = fabs(v); /* complex_abs of (v, 0) */
        }
        int dx = 0, dy = 0;
        orc_xcorr_displacement(ref_frame, absf, ncols, nrows, &dx, &dy, NULL);
        if (shifts) {
            shifts[2 * f] = dx;
            shifts[2 * f + 1] = dy;
        }
        orc_shifted(absf, shf, ncols, nrows, -dx, -dy);
        for (long n = 0; n < np; ++n)
            sum_acc[n] += shf[n];
        orc_fft_2d(indata, nrows, ncols, -1);
        orc_accumulate_f32(bispec32, indata, ncols, nrows, depth, nthreads);
        for (long n = 0; n < np; ++n)
            powerspec_acc[n] += cnorm(indata[2 * n], indata[2 * n + 1]);
    }
    free(indata);
    free(absf);
    free(shf);
    return 0;
}

int orc_run_stack(const void* frames, int dtype, long nframes, long ncols, long nrows,
                  long depth, double reco_radius, int fp64_bispec, int nthreads,
                  int* shifts, double* sumarray, double* powerspec,
                  float* bispec32, double* bispec64,
                  double* phases, unsigned char* flags, double* consistency,
                  double* image)
{
    if (nframes < 1 || ncols < 1 || nrows < 1)
        return -2;
    const long np = ncols * nrows;
    orc_bispec_desc d;
    orc_bispec_describe(ncols, nrows, depth, depth, &d);
    float* b32 = NULL;
    double* b64 = NULL;
    if (fp64_bispec)
        b64 = (double*)calloc((size_t)d.base_size * 2, sizeof(double));
    else
        b32 = (float*)calloc((size_t)d.base_size * 2, sizeof(float));
    double* indata = (double*)malloc(sizeof(double) * 2 * (size_t)np);
    double* pw = (double*)calloc((size_t)np, sizeof(double));   /* real parts of powerspec */
    double* sum = (double*)calloc((size_t)np, sizeof(double));
    double* ref = (double*)malloc(sizeof(double) * (size_t)np);
    double* absf = (double*)malloc(sizeof(double) * (size_t)np);
    double* shf = (double*)malloc(sizeof(double) * (size_t)np);

    for (long f = 0; f < nframes; ++f) {
        for (long n = 0; n < np; ++n) {
            const double v = pixel(frames, dtype, f * np + n);
            indata[2 * n] = v;
            indata[2 * n + 1] = 0.0;
        }
        if (f == 0) {
            /* main.cpp:263-268: sum = real(frame 0), reference = copy of it */
            for (long n = 0; n < np; ++n) {
                sum[n] = indata[2 * n];
                ref[n] = sum[n];
            }
            if (shifts) {
                shifts[0] = 0;
                shifts[1] = 0;
            }
        } else {
            /* main.cpp:289-294 */
            for (long n = 0; n < np; ++n)
                absf[n] = fabs(indata[2 * n]);
            int dx = 0, dy = 0;
            orc_xcorr_displacement(ref, absf, ncols, nrows, &dx, &dy, NULL);
            if (shifts) {
                shifts[2 * f] = dx;
                shifts[2 * f + 1] = dy;
            }
            orc_shifted(absf, shf, ncols, nrows, -dx, -dy);
            for (long n = 0; n < np; ++n)
                sum[n] += shf[n];
        }
        orc_fft_2d(indata, nrows, ncols, -1);                         /* main.cpp:271, 296 */
        if (b32)
            orc_accumulate_f32(b32, indata, ncols, nrows, depth, nthreads);
        else
            orc_accumulate_f64(b64, indata, ncols, nrows, depth, nthreads);
        for (long n = 0; n < np; ++n)                                 /* main.cpp:274-279, 300-305 */
            pw[n] += cnorm(indata[2 * n], indata[2 * n + 1]);
    }
    /* main.cpp:307-312 */
    const double nf = (double)nframes;
    for (long n = 0; n < np; ++n)
        sum[n] = sum[n] / nf;
    const double pnorm = (double)((size_t)nframes * (size_t)np);
    for (long n = 0; n < np; ++n)
        pw[n] = pw[n] / pnorm;
    if (b32) {
        const float fnf = (float)nframes;
        for (long n = 0; n < 2 * d.base_size; ++n)
            b32[n] = b32[n] / fnf;
    } else {
        for (long n = 0; n < 2 * d.base_size; ++n)
            b64[n] = b64[n] / nf;
    }
    if (sumarray)
        memcpy(sumarray, sum, sizeof(double) * (size_t)np);
    if (powerspec)
        for (long n = 0; n < np; ++n) {
            powerspec[2 * n] = pw[n];
            powerspec[2 * n + 1] = 0.0;
        }
    if (bispec32 && b32)
        memcpy(bispec32, b32, sizeof(float) * 2 * (size_t)d.base_size);
    if (bispec64 && b64)
        memcpy(bispec64, b64, sizeof(double) * 2 * (size_t)d.base_size);

    /* main.cpp:318-319 */
    double* ph = (double*)malloc(sizeof(double) * 2 * (size_t)np);
    unsigned char* fl = (unsigned char*)malloc((size_t)np);
    double* cs = (double*)malloc(sizeof(double) * (size_t)np);
    int rc = orc_reconstruct_phases(b32, b64, ncols, nrows, depth, reco_radius, ph, fl, cs);
    if (rc == 0) {
        if (phases)
            memcpy(phases, ph, sizeof(double) * 2 * (size_t)np);
        if (flags)
            memcpy(flags, fl, (size_t)np);
        if (consistency)
            memcpy(consistency, cs, sizeof(double) * (size_t)np);
        if (image) {
            /* main.cpp:329-346 */
            double* win = (double*)malloc(sizeof(double) * (size_t)np);
            orc_general_hamming(win, ncols, nrows, reco_radius * 2.0, 0.5);
            for (long n = 0; n < np; ++n) {
                const double s = sqrt(pw[n]);
                /* phases *= window (complex (w,0)); result = (s,0) * phases */
                const double wr = ph[2 * n] * win[n] - ph[2 * n + 1] * 0.0;
                const double wi = ph[2 * n] * 0.0 + ph[2 * n + 1] * win[n];
                image[2 * n] = s * wr - 0.0 * wi;
                image[2 * n + 1] = s * wi + 0.0 * wr;
            }
            orc_fft_2d(image, nrows, ncols, +1);
            /* main.cpp:371-376: divide by the largest |.| */
            double mx = 0.0;
            for (long n = 0; n < np; ++n) {
                const double a = hypot(image[2 * n], image[2 * n + 1]);
                if (n == 0 || mx < a)
                    mx = a;
            }
            for (long n = 0; n < 2 * np; ++n)
                image[n] = image[n] / mx;
            free(win);
        }
    }
    free(ph);
    free(fl);
    free(cs);
    free(b32);
    free(b64);
    free(indata);
    free(pw);
    free(sum);
    free(ref);
    free(absf);
    free(shf);
    return rc;
}
