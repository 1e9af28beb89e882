/*
 * fftw3.h -- project-written stand-in exposing the FFTW3 API names that the
 * reference's hot path calls (include/crosscorrel.h:112-141,
 * smip-cli/main.cpp:256-259, 340-346).  FFTW3 is not installed here; the
 * transforms are the oracle's own double-precision FFT (oracle/smip_oracle.c).
 * TEST INFRASTRUCTURE: only the oracle/ref build of the reference uses it.
 */
#ifndef SMIP_FFTW3_STANDIN_H
#define SMIP_FFTW3_STANDIN_H
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct smip_fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
#endif
