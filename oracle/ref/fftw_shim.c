/*
 * fftw_shim.c -- implementation of the FFTW3 API stand-in (oracle/ref/fftw3.h)
 * on top of the oracle's FFT.  Plans only record their arguments; execution is
 * unnormalised like FFTW.  TEST INFRASTRUCTURE.
 */
#include "fftw3.h"
#include "../smip_oracle.h"

#include <stdlib.h>
#include <string.h>

enum { K_C2C = 0, K_R2C = 1, K_C2R = 2 };

struct smip_fftw_plan_s {
    int kind, n0, n1, sign;
    void* in;
    void* out;
};

static fftw_plan mk(int kind, int n0, int n1, void* in, void* out, int sign)
{
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->kind = kind;
    p->n0 = n0;
    p->n1 = n1;
    p->in = in;
    p->out = out;
    p->sign = sign;
    return p;
}

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags)
{
    (void)flags;
    return mk(K_C2C, n0, n1, in, out, sign);
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags)
{
    (void)flags;
    return mk(K_R2C, n0, n1, in, out, -1);
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags)
{
    (void)flags;
    return mk(K_C2R, n0, n1, in, out, +1);
}

void fftw_execute(const fftw_plan p)
{
    const long n = (long)p->n0 * p->n1;
    switch (p->kind) {
    case K_C2C:
        if (p->out != p->in)
            memcpy(p->out, p->in, sizeof(double) * 2 * (size_t)n);
        orc_fft_2d((double*)p->out, p->n0, p->n1, p->sign);
        break;
    case K_R2C:
        orc_fft_r2c_2d((const double*)p->in, (double*)p->out, p->n0, p->n1);
        break;
    default:
        orc_fft_c2r_2d((const double*)p->in, (double*)p->out, p->n0, p->n1);
        break;
    }
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
