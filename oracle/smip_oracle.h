/*
 * smip_oracle.h -- CPU oracle for the speckle-masking (SMIP) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (hangeza/speckle-stacker v0.3.2) used as the checker for the CUDA
 * library.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm may load it.  The product path never calls into this code.
 *
 * Parity is pinned two ways: against fixtures produced by the reference's own
 * headers compiled in place (oracle/ref/, tests/golden/), and against the
 * reference's own unit-test vectors (tests/bispectrum_test.cpp,
 * tests/correl_test.cpp).
 *
 * Conventions (same as the reference):
 *   - 2-D arrays are row-major, x (column) fastest: a[x + y*ncols]
 *     (include/array2.h:310-339).  Signed indices wrap by +size when negative.
 *   - complex values are interleaved (re, im) pairs.
 *   - The packed bispectrum uses the reference's half-space layout
 *     (include/bispectrum.h:203-220, 324-349).
 */
#ifndef SMIP_ORACLE_H
#define SMIP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- bispectrum descriptor: include/bispectrum.h:143-160, 203-220 ---- */
typedef struct {
    long dimsizes[4];   /* {ncols, nrows, depth, depth} as passed to the ctor */
    long sizes[4];      /* (d/2)*2+1 */
    long base_sizes[4]; /* sizes - sizes*{1,0,1,0}/2 */
    long base_size;
    long totalsize;
    int min_idx[4];
    int max_idx[4];
} orc_bispec_desc;

void orc_bispec_describe(long ncols, long nrows, long d2, long d3, orc_bispec_desc* d);
/* include/bispectrum.h:324-349 (no range check, silent wrap) */
long orc_calc_offset(const orc_bispec_desc* d, const int idx[4]);
/* include/bispectrum.h:280-316 */
void orc_calc_indices(const orc_bispec_desc* d, long addr, int idx[4]);
/* include/bispectrum.h:482-512 (+553-589, 162-174).  Returns the packed
 * offset, sets *conj; returns -1 where the reference throws out_of_range. */
long orc_get_element_offset(const orc_bispec_desc* d, const int idx[4], int* conj);

/* ---- FFT (stand-in for FFTW3, double precision, unnormalised) ---- */
/* sign = -1 forward (FFTW_FORWARD), +1 backward (FFTW_BACKWARD) */
void orc_fft_2d(double* data, long nrows, long ncols, int sign);
/* FFTW r2c 2-D layout: out is nrows x (ncols/2+1) complex */
void orc_fft_r2c_2d(const double* in, double* out, long nrows, long ncols);
/* FFTW c2r 2-D layout: in is nrows x (ncols/2+1) complex (not modified) */
void orc_fft_c2r_2d(const double* in, double* out, long nrows, long ncols);

/* ---- bispectrum accumulation: include/bispectrum.h:356-409 ----
 * fft: ncols x nrows complex<double> spectrum in FFT order.
 * B:   packed bispectrum, base_size complex values.
 * _f32 narrows the spectrum to complex<float> first (Bispectrum<complex<float>>,
 * the reference as shipped); _f64 keeps double (the FP64 oracle).
 * nthreads > 1 splits the u_x loop across threads; each packed element is
 * written by exactly one thread, so results do not depend on nthreads. */
void orc_accumulate_f32(float* B, const double* fft, long ncols, long nrows, long depth, int nthreads);
void orc_accumulate_f64(double* B, const double* fft, long ncols, long nrows, long depth, int nthreads);

/* ---- closure-phase recovery: include/phasereco.h:33-123, src/phasereco.cpp:17-36 ---- */
void orc_next_reco_index(double* r, double* phi, int* i, int* j);
/* Number of visits the reconstruct_phases loop makes for this radius and
 * (if out != NULL and cap large enough) the visited (i,j) pairs. */
long orc_reco_visits(double reco_radius, int* out_ij, long cap);
/* B is the packed bispectrum as complex<float> (bf32) or complex<double> (bf64);
 * exactly one of them is non-NULL.  phases: xsize*ysize complex<double>;
 * flags: xsize*ysize bytes; consistency: xsize*ysize doubles (may be NULL).
 * Returns 0, or -1 where the reference would throw out_of_range. */
int orc_reconstruct_phases(const float* bf32, const double* bf64,
                           long xsize, long ysize, long depth, double reco_radius,
                           double* phases, unsigned char* flags, double* consistency);

/* ---- cross correlation: include/crosscorrel.h:96-179 ----
 * ref, frame: ncols x nrows real.  corr (optional) receives the correlation. */
void orc_xcorr_displacement(const double* ref, const double* frame, long ncols, long nrows,
                            int* dx, int* dy, double* corr);

/* ---- Array2::shifted: include/array2.h:603-622 ---- */
void orc_shifted(const double* in, double* out, long ncols, long nrows, int dx, int dy);

/* ---- GeneralHamming / Hann: include/window_function.h:70-85 ---- */
void orc_general_hamming(double* out, long xsize, long ysize, double aperture, double alpha);

/* ---- output mapping: Array2Mat (include/videoio.h:100-156) ----
 * mapToColor<uint16_t> (include/videoio.h:178-206): n values, clamped to
 * [0, 1], to 16-bit (r, g, b) triples, 3*n values written as r, g, b (the
 * PNG order of the reference's BGR cv::Mat).  A NaN value maps as 0. */
void orc_map_to_color_u16(const double* v, long n, uint16_t* rgb);
/* Array2Mat's pixel order (videoio.h:137-146): pixel (x, y) of the output
 * shows element (x + min_x, y + min_y) of the signed index range when
 * signed_symmetry is set (an fftshift), element (x, y) otherwise. */
void orc_array2mat_order(const double* in, double* out, long ncols, long nrows, int signed_symmetry);

/* ---- whole pipeline: smip-cli/main.cpp:246-378 (without OpenCV) ----
 * frames: nframes frames, ncols x nrows, dtype 0=u8 1=u16 2=f32 3=f64,
 *         frame stride = ncols*nrows elements.
 * fp64_bispec: 0 = Bispectrum<complex<float>> (reference), 1 = complex<double>.
 * Outputs (any may be NULL):
 *   shifts      2*nframes ints (frame 0 gets 0,0)
 *   sumarray    ncols*nrows doubles, normalised (main.cpp:308)
 *   powerspec   ncols*nrows complex doubles, normalised (main.cpp:310)
 *   bispec32 / bispec64  base_size complex, normalised (main.cpp:312)
 *   phases      ncols*nrows complex doubles (pre-window, as reconstructed)
 *   flags, consistency  phase map
 *   image       ncols*nrows complex doubles, normalised by max |.| (main.cpp:375-376)
 * Returns 0 on success. */
int orc_run_stack(const void* frames, int dtype, long nframes, long ncols, long nrows,
                  long depth, double reco_radius, int fp64_bispec, int nthreads,
                  int* shifts, double* sumarray, double* powerspec,
                  float* bispec32, double* bispec64,
                  double* phases, unsigned char* flags, double* consistency,
                  double* image);

/* Per-frame part of the pipeline only (main.cpp:263-306): FFT, bispectrum,
 * power spectrum, cross correlation and shift-and-add for nframes frames,
 * continuing from the given accumulators.  Used for bounded timing samples. */
int orc_accumulate_frames(const void* frames, int dtype, long nframes, long ncols, long nrows,
                          long depth, int nthreads, const double* ref_frame,
                          float* bispec32, double* powerspec_acc, double* sum_acc, int* shifts);

#ifdef __cplusplus
}
#endif
#endif
