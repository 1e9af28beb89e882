/*
 * smip_gpu.h -- C ABI of the GB300 speckle-masking (SMIP) engine.
 *
 * libsmip_gpu.so replaces the hot path of hangeza/speckle-stacker v0.3.2
 * (per-frame FFT + power spectrum, bispectrum accumulation, cross-correlation
 * shift-and-add, closure-phase recovery, final reconstruction).  All entry
 * points are extern "C", take plain pointers and sizes, return an int status
 * (SMIP_OK = 0) and leave a thread-local message for smip_last_error().
 * The C++ layer in speckle-stacker_gb300/include/smip/gpu.hpp maps the status
 * codes back to the exception types the reference throws.
 *
 * Conventions (the reference's own):
 *   - 2-D arrays are ncols x nrows, row-major, x fastest; spectra, phases and
 *     power spectra are in FFT order (negative frequencies wrapped by +size,
 *     include/array2.h:310-339).
 *   - complex values are interleaved (re, im): complex<float> bispectrum
 *     (include/types.h:33), complex<double> phases/images (types.h:32).
 *   - the bispectrum is the reference's packed half-space array, base_size =
 *     (ncols/2+1)((nrows/2)*2+1)(d/2+1)(d+1) elements, d = bdepth rounded
 *     down to even (include/bispectrum.h:203-220, 324-349).
 *
 * Every call is asynchronous on the object's CUDA stream unless it returns
 * host data; host-data calls synchronise that stream first.
 */
#ifndef SMIP_GPU_H
#define SMIP_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SMIP_GPU_API __attribute__((visibility("default")))
#else
#define SMIP_GPU_API
#endif

/* ---- status codes (mirroring the reference's exception types) ------------ */
#define SMIP_OK 0
#define SMIP_E_INVALID_ARGUMENT 1 /* std::invalid_argument (crosscorrel.h:100-102, bispectrum.h:235-237) */
#define SMIP_E_OUT_OF_RANGE 2     /* std::out_of_range (bispectrum.h:491-507, array2.h:274-306) */
#define SMIP_E_RUNTIME 3          /* std::runtime_error (I/O bispectrum.h:418-459, /0 array_base.h:342-344) */
#define SMIP_E_DOMAIN 4           /* std::domain_error (window aperture <= 0, window_function.h:20) */
#define SMIP_E_BAD_CALL 5         /* std::bad_function_call (correlation not ready, crosscorrel.h:149-159) */
#define SMIP_E_NO_MEMORY 6        /* device allocation failed or admission budget exceeded */
#define SMIP_E_CUDA 7             /* CUDA runtime error */
#define SMIP_E_TIMEOUT 8          /* a bounded device-side wait expired (kernel returned early) */
#define SMIP_E_UNSUPPORTED 9      /* shape outside what the GPU kernels implement */

/* ---- frame element types ------------------------------------------------- */
#define SMIP_U8 0
#define SMIP_U16 1
#define SMIP_F32 2
#define SMIP_F64 3

typedef struct smip_stack* smip_stack_t;

/* Message for the last failing call on this thread ("" if none). */
SMIP_GPU_API const char* smip_last_error(void);

/* Library version; the reference's is config/config.h:40-46 (0.3.2). */
SMIP_GPU_API int smip_version(int* major, int* minor, int* patch);

/* ========================================================================== *
 * Stack: one speckle-masking job.  Owns the device-resident accumulators of
 * smip-cli/main.cpp:232-312 -- packed bispectrum plus Kahan compensation
 * (Bispectrum<complex<float>>, main.cpp:253), power spectrum (main.cpp:274-279,
 * 300-305), shift-and-add sum (main.cpp:263-266, 293-294), the cross
 * correlation reference (frame 0, main.cpp:268) and the frame count.
 * ========================================================================== */

/* Replaces Bispectrum<complex<float>>({ncols, nrows, bdepth, bdepth})
 * (bispectrum.h:183-192, main.cpp:253) plus the accumulators above.
 * stream: a cudaStream_t to run on, or NULL for a stream owned by the stack.
 * batch_frames: frames per accumulation batch (0 = library default).
 * Supported: any ncols, nrows in [3, 1024] (powers of two in [16, 512] run
 * radix-2 transforms, every other size mixed-radix ones, as FFTW plans any
 * size for the reference, main.cpp:256-259); bdepth/2*2 in [2, 64] and
 * < min(ncols, nrows). */
SMIP_GPU_API int smip_stack_create(smip_stack_t* out, int device, long ncols, long nrows,
                                   long bdepth, void* stream, long batch_frames);
SMIP_GPU_API int smip_stack_destroy(smip_stack_t s);

/* Replaces the per-frame body of smip-cli/main.cpp:281-306 (and 247-279 for
 * the stack's first frame): cross-correlate against frame 0 (crosscorrel.h:
 * 181-189), add the back-shifted frame to the sum (array2.h:603-622), forward
 * FFT (main.cpp:296), accumulate the bispectrum (bispectrum.h:356-409) and the
 * power spectrum.  frames: count frames of ncols x nrows elements of dtype,
 * consecutive frames frame_stride_bytes apart (0 = tightly packed); on_device
 * non-zero if the pointer is device memory.  Host buffers are read before the
 * call returns unless they are page-locked, in which case they must stay
 * unchanged until smip_stack_sync. */
SMIP_GPU_API int smip_stack_push_frames(smip_stack_t s, const void* frames, int dtype, long count,
                                        long frame_stride_bytes, int on_device);

/* Tuning of the stack's bispectrum kernel (no counterpart in the reference):
 * variant 0 stages four frames per shared-memory ring stage, 1 two;
 * min_part_frames is the fewest frames a split part of a last-wave tile gets
 * (0 = 8; a batch's last partial wave of tiles is split by frames so that it
 * fills the GPU).  Neither changes which triples are summed; the split
 * changes the order of a tile's partial sums, so results stay within the
 * parity tolerances and a stack with the same settings gives the same bits.
 * smip_gb300.autotune picks both per shape. */
SMIP_GPU_API int smip_stack_set_kernel_config(smip_stack_t s, int variant, int min_part_frames);

/* Phase-recovery estimator for smip_stack_reconstruct / smip_stack_finish.
 * SMIP_RECO_SPIRAL (default): the reference's walk (phasereco.h:33-123), each
 * point from every pair whose phases exist when the spiral reaches it.
 * SMIP_RECO_RINGS: not the reference's estimator -- the points of one turn of
 * the spiral (a ring) are formed in parallel from the pairs set in earlier
 * rings only; faster, and its phases differ from the reference's (the
 * difference is measured, not bounded by it). */
#define SMIP_RECO_SPIRAL 0
#define SMIP_RECO_RINGS 1
SMIP_GPU_API int smip_stack_set_reco_mode(smip_stack_t s, int mode);

/* Replaces Bispectrum::accumulate_from_fft(const Array2<complex<double>>&)
 * (bispectrum.h:82-83, 356-409) for spectra computed elsewhere: count spectra
 * of ncols x nrows complex<double> in FFT order, host or device memory.
 * Only the bispectrum is accumulated (no power spectrum or shift-and-add). */
SMIP_GPU_API int smip_stack_accumulate_fft(smip_stack_t s, const double* spectra, long count, int on_device);

/* Zeroes the accumulators and the frame count, keeping the device buffers,
 * so the stack can take a new job (no counterpart in the reference, whose
 * accumulators live for one smip-cli run). */
SMIP_GPU_API int smip_stack_reset(smip_stack_t s);

/* Runs the pending partial batch; smip_stack_sync also waits for it. */
SMIP_GPU_API int smip_stack_flush(smip_stack_t s);
SMIP_GPU_API int smip_stack_sync(smip_stack_t s);

/* Runs the pending (staged, not yet launched) frame batches of count stacks:
 * each stack's per-frame kernels on its own stream, then the bispectrum work
 * of all of them -- any frame sizes and depths -- as ONE persistent launch
 * over a device work list of every stack's tiles, longest first.  That launch
 * is a CUDA graph captured once (its stack records and work list are copied
 * into device memory by the graph itself; it is captured again only when its
 * buffers grow).  Stacks without pending frames are skipped; all must live on
 * one device and appear once.  Later calls on each stack are ordered after
 * the launch.  The results are bit-identical to smip_stack_flush on each
 * stack.  No counterpart in the reference, which accumulates one stack per
 * smip-cli run (main.cpp:281-312); the serving loop uses it. */
SMIP_GPU_API int smip_batch_launch(smip_stack_t* stacks, long count);

/* smip_batch_launch with reserve_sms streaming multiprocessors left out of
 * the persistent grid (0 <= reserve_sms < SM count; 0 is smip_batch_launch),
 * so that phase recoveries of stacks launched earlier -- one block each, on
 * their high-priority streams -- run beside the launch instead of after it.
 * One graph is kept per grid size.  Results do not depend on reserve_sms. */
SMIP_GPU_API int smip_batch_launch_reserve(smip_stack_t* stacks, long count, int reserve_sms);

/* Diagnostic of the failure path: runs a kernel whose two waits (an mbarrier
 * nothing arrives on, a device flag nothing sets) can never be satisfied.
 * Both give up after timeout_s seconds (at most 10), record the expiry and
 * return, so the call returns SMIP_E_TIMEOUT -- what any call reports after a
 * bounded device wait expired -- and the device stays usable.  No counterpart
 * in the reference (its loops are host code). */
SMIP_GPU_API int smip_diag_bounded_wait(int device, double timeout_s);

SMIP_GPU_API int smip_stack_frame_count(smip_stack_t s, long* nframes);
SMIP_GPU_API int smip_stack_bispectrum_size(smip_stack_t s, long* base_size);

/* Integer shift-and-add shifts of frames [first, first+count): (x, y) pairs
 * as CrossCorrelation::operator() returns them (crosscorrel.h:166-179);
 * frame 0 is the reference and reports (0, 0). */
SMIP_GPU_API int smip_stack_shifts(smip_stack_t s, int* xy, long first, long count);

/* Normalised results of main.cpp:307-312, copied to host:
 * sum: ncols*nrows doubles (sumarray / nframes);
 * power: ncols*nrows doubles (real part of powerspec / (nframes*ncols*nrows));
 * bispec: 2*base_size floats (bispectrum / nframes, the bispectrum.dat payload). */
SMIP_GPU_API int smip_stack_sum(smip_stack_t s, double* sum);
SMIP_GPU_API int smip_stack_power(smip_stack_t s, double* power);
SMIP_GPU_API int smip_stack_bispectrum(smip_stack_t s, float* bispec);

/* Replaces reconstruct_phases<complex_t, complex<float>>(bispectrum, ncols,
 * nrows, reco_radius, &pm) (phasereco.h:16-19, 33-123) on the stack's
 * normalised bispectrum.  phases: ncols*nrows complex<double>; flags and
 * consistency: the PhaseMap (phasemap.h:10-18), ncols*nrows each.  Any
 * output pointer may be NULL.  SMIP_E_OUT_OF_RANGE where the reference's
 * Bispectrum::get_element would throw. */
SMIP_GPU_API int smip_stack_reconstruct(smip_stack_t s, double reco_radius, double* phases,
                                        unsigned char* flags, double* consistency);

/* Replaces main.cpp:318-376 as a whole: phase reconstruction, Hann window of
 * aperture 2*reco_radius (window_function.h:39-46, main.cpp:329-330),
 * sqrt(power) x phases, backward FFT and division by the largest modulus.
 * image: ncols*nrows complex<double> (may be NULL); phases/flags/consistency
 * as above (pre-window phases, as reconstruct_phases returns them). */
SMIP_GPU_API int smip_stack_finish(smip_stack_t s, double reco_radius, double* image, double* phases,
                                   unsigned char* flags, double* consistency);

/* Allocates the reconstruction's device buffers and builds its spiral visit
 * tables for reco_radius ahead of smip_stack_reconstruct / smip_stack_finish
 * (which otherwise do it on their first call, and again for a new radius):
 * a serving loop prepares its pooled stacks so that no job allocates device
 * memory.  Results do not change.  No counterpart in the reference. */
SMIP_GPU_API int smip_stack_prepare_reco(smip_stack_t s, double reco_radius);

/* Adds src's accumulators into dst (same shape): frame-level sharding of one
 * stack across accumulators (the accumulation is additive).  dst keeps its
 * own reference frame; src must have been created after dst received its
 * first frame and with dst as reference (smip_stack_share_reference). */
SMIP_GPU_API int smip_stack_merge(smip_stack_t dst, smip_stack_t src);
/* Makes src correlate against dst's reference frame (frame 0 of dst). */
SMIP_GPU_API int smip_stack_share_reference(smip_stack_t dst, smip_stack_t src);

/* Bispectrum::write_to_file (bispectrum.h:411-430): the normalised
 * bispectrum in the reference's bispectrum.dat format. */
SMIP_GPU_API int smip_stack_save_bispectrum(smip_stack_t s, const char* path);

/* Bispectrum::read_from_file (bispectrum.h:432-462) into an empty stack of the
 * same shape: the accumulator resumes as the file's (normalised) bispectrum
 * times nframes (0 = 1) with zero compensation, so smip_stack_reconstruct runs
 * on it and smip_stack_accumulate_fft can add further spectra (a stack needs
 * its reference frame for frames, so smip_stack_push_frames is refused).
 * SMIP_E_RUNTIME on I/O errors, SMIP_E_INVALID_ARGUMENT on a shape mismatch. */
SMIP_GPU_API int smip_stack_load_bispectrum(smip_stack_t s, const char* path, long nframes);

/* Whole-stack checkpoint of a served job (no counterpart in the reference,
 * whose only persistence is bispectrum.dat): after a flush, the accumulators
 * (bispectrum and its compensation, power spectrum, shift-and-add sum), the
 * shifts so far and the reference frame with its spectrum.  Loading it into an
 * empty stack of the same shape resumes the job: frames pushed afterwards give
 * what pushing them into the original stack would have given. */
SMIP_GPU_API int smip_stack_save_state(smip_stack_t s, const char* path);
SMIP_GPU_API int smip_stack_load_state(smip_stack_t s, const char* path);

/* smip_stack_load_bispectrum from memory: bispec holds base_size normalised
 * complex<float> in the packed layout smip_stack_bispectrum returns (the data
 * block of bispectrum.dat, bispectrum.h:442-461); the stack must be empty. */
SMIP_GPU_API int smip_stack_set_bispectrum(smip_stack_t s, const float* bispec, long nframes);

/* ========================================================================== *
 * Standalone calls mirroring the reference's free functions and classes.
 * ========================================================================== */

/* reconstruct_phases on a host Bispectrum<complex<float>> (phasereco.h:16-19).
 * bispec: 2*base_size floats for (xsize, ysize, bdepth). */
SMIP_GPU_API int smip_reconstruct_phases(int device, const float* bispec, long xsize, long ysize, long bdepth,
                                         double reco_radius, double* phases, unsigned char* flags,
                                         double* consistency);

/* NextRecoIndex (phasereco.h:21, phasereco.cpp:17-36); host arithmetic. */
SMIP_GPU_API int smip_next_reco_index(double* r, double* phi, int* i, int* j);

/* Number of visits of the reconstruction loop for reco_radius and, when
 * ij != NULL, the visited (i, j) pairs (phasereco.h:56-68); host arithmetic. */
SMIP_GPU_API int smip_reco_visits(double reco_radius, int* ij, long cap, long* count);

/* CrossCorrelation<double>::get_displacement(ref, frame) (crosscorrel.h:54-58)
 * on the GPU: ref and frame are ncols x nrows doubles (host).  corr (may be
 * NULL) receives the unnormalised correlation array (crosscorrel.h:147-152). */
SMIP_GPU_API int smip_xcorr_displacement(int device, const double* ref, const double* frame, long ncols,
                                         long nrows, int* dx, int* dy, double* corr);

/* Same shift as smip_xcorr_displacement, for callers that cannot allocate
 * device memory while they run: acquisition loops that fix their buffers at
 * start-up (a cudaMalloc can stall the device mid-stream) and plug-ins whose
 * host application owns device memory through its own pool allocator.  No
 * counterpart in the reference.  ref, frame: device pointers to ncols x nrows
 * doubles; shift: device pointer to two ints (x, y), written on `stream`
 * (a cudaStream_t, or NULL for the default stream).  Allocates nothing: all
 * intermediates live in one fixed ~3 MB device array inside the library, so
 * ncols and nrows must be powers of two in [16, 256] (SMIP_E_UNSUPPORTED
 * otherwise).  The first call on a device looks up that array and uploads
 * constants, so make it before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race and must be ordered by the caller. */
SMIP_GPU_API int smip_xcorr_displacement_noalloc(const double* ref, const double* frame, long ncols, long nrows,
                                                 int* shift, void* stream);

/* Array2<double>::shifted(DimVector<int,2>{dx, dy}) (array2.h:603-622) on the
 * GPU: out(x, y) = in(x - dx, y - dy), zero where that lies outside; ncols x
 * nrows doubles, row-major, host memory.  |dx| >= ncols or |dy| >= nrows is
 * SMIP_E_OUT_OF_RANGE: the reference's clamped copy range reads outside the
 * array there.  The stack pipeline fuses this shift into its shift-and-add. */
SMIP_GPU_API int smip_shifted(int device, const double* in, double* out, long ncols, long nrows, int dx, int dy);

/* Hann<double>(xsize, ysize, aperture) (window_function.h:39-46, 70-85),
 * computed on the GPU; SMIP_E_DOMAIN for aperture <= 0. */
SMIP_GPU_API int smip_hann(int device, double* out, long xsize, long ysize, double aperture);

/* Instrumentation (no counterpart in the reference).
 * smip_stack_set_timing: record CUDA events around every bispectrum-kernel
 * launch on the stack's stream.  smip_stack_kernel_time: the summed kernel
 * time (ms), launches and frames since the last query (waits for the stream).
 * smip_kernel_launches: kernels this library has launched in this process. */
SMIP_GPU_API int smip_stack_set_timing(smip_stack_t s, int on);
SMIP_GPU_API int smip_stack_kernel_time(smip_stack_t s, double* bispec_ms, long* launches, double* frames);
SMIP_GPU_API long long smip_kernel_launches(void);

/* The device's copy of Bispectrum::get_element's index path (bispectrum.h:
 * 482-512, 553-589, 324-349) for n tuples idx[4*q..4*q+3] = (ux, uy, vx, vy):
 * off[q] = packed offset (-1 where the reference throws out_of_range), conj[q]
 * = 1 where the element is returned conjugated.  The phase-recovery kernel
 * uses exactly this function; it is exported so its parity can be checked. */
SMIP_GPU_API int smip_bispec_offsets(int device, long ncols, long nrows, long bdepth, const int* idx, long n,
                                     long long* off, int* conj);

#ifdef __cplusplus
}
#endif
#endif /* SMIP_GPU_H */
