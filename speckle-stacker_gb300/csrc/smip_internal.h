// smip_internal.h -- declarations shared by the SMIP host runtime and kernels.
#pragma once

#include <vector>

#include <cstdint>
#include <cuda_runtime.h>
#include <string>

namespace smip_gpu {

// device-side error codes written to a stack's error word
enum : int {
    SMIP_DEV_OK = 0,
    SMIP_DEV_ERR_TIMEOUT = 1,      // a bounded mbarrier wait expired
    SMIP_DEV_ERR_OUT_OF_RANGE = 2, // Bispectrum::get_element would throw
};

constexpr int kMaxLog = 9;        // radix-2 kernels: frames up to 512 x 512
constexpr int kTwLog = kMaxLog;   // twiddle table for length 2^kTwLog
constexpr int kMaxSide = 1024;    // any frame side up to this (mixed-radix kernels, k_fftg.cu)
constexpr int kMaxFactors = 16;

// Factorisation of one transform length for the mixed-radix kernels.
struct GenPlan {
    int L;
    int nf;
    int fac[kMaxFactors];
    // per pass f and output o: j | e0 << 16, the pass's input index and twiddle
    // exponent step (k_fftg.cu), nf x L entries in device memory (null: computed)
    const unsigned* map = nullptr;
};
GenPlan make_gen_plan(int L);
constexpr int kRowBlock = 16;     // rows per CTA in the row passes
constexpr int kColLines = 8;      // frames per FFT pass in the column kernel

// Geometry of one stack (all derived from ncols = W, nrows = H, depth).
struct Geometry {
    int W, H;         // frame size
    int logW, logH;   // radix-2 path: log2 of W and H
    bool generic;     // W or H not a power of two in [16, 512]: mixed-radix kernels
    int hw;           // W/2 + 1: u_x half-plane rows a = -x in [0, W/2]
    int Hs;           // row pitch of the spectra S (H rounded up to even: 16-byte TMA strides)
    int bs1;          // packed bispectrum extent of u_y: (H/2)*2 + 1 (bispectrum.h:203-220)
    int De;           // bispectrum depth rounded down to even
    int E;            // packed elements per (u_x, u_y): (De/2+1)(De+1)
    long long base_size;
    GenPlan pW, pH;   // generic path: factorisations of W and H
};


// float-float complex value hi + lo (forward-FFT intermediates, twiddles)
struct dfc {
    float2 h, l;
};
// Twiddle tables of one transform length L (generic path): exp(-2 pi i k / L), k < L.
struct GenTw {
    dfc* df = nullptr;
    float2* f32 = nullptr;
    double2* f64 = nullptr;
    unsigned* map = nullptr; // GenPlan::map of this length
};

// Every kernel launch site reports itself here (process-wide counter).
void note_launches(int n);

// Sets the message smip_last_error() returns on this thread.
void set_error_message(const std::string& m);

// ---------------------------------------------------------------- launchers
// All launchers are asynchronous on `st` and return cudaGetLastError().

// frames (dtype) -> G'(a, y) = sum_x f(x,y) exp(+2 pi i a x / W), float-float,
// stored [f][a][y].  dtype: 0 u8, 1 u16, 2 f32, 3 f64.  copy_out (optional,
// device memory): the frames as read, same stride.
cudaError_t launch_row_pass(int dtype, const void* frames, long long frame_stride_elems, int nframes,
                            const Geometry& g, dfc* Gt, const dfc* twdf, cudaStream_t st, void* copy_out = nullptr);

// Column pass.  mode 1: frame 0 only -> Rout (the reference spectrum).
// mode 0: S[f][a][c] = F(-a, c - H/2), power partials, and the FP32 inverse
// column FFT of conj(R)·F for the cross correlation into T[f][a][y].
cudaError_t launch_col_pass(int mode, const dfc* Gt, float2* S, const float2* Rbuf, float2* Rout, float2* T,
                            double* Ppart, int nframes, int frames_per_chunk, int skip_xcorr_frame0,
                            const Geometry& g, const dfc* twdf, const float2* tw, cudaStream_t st);
cudaError_t launch_power_reduce(double* P, const double* Ppart, int nchunks, const Geometry& g, cudaStream_t st);

// Row pass of the correlation's inverse transform: corr[f][y][x] (float).
// corr: [nframes][H][W] correlation; rowmax: [nframes][H] maximum of each row
cudaError_t launch_xcorr_rows(const float2* T, float* corr, float* rowmax, int nframes, const Geometry& g,
                              const float2* tw, cudaStream_t st);

// Integer shift per frame: FP32 correlation peak, candidates re-scored exactly.
// ref_sq: sum of squares of the reference frame (double, device).
cudaError_t launch_xcorr_shift(int dtype, const float* corr, const float* rowmax, const void* frames,
                               long long frame_stride_elems, const void* ref, const double* ref_sq, int nframes,
                               int first_is_frame0, const Geometry& g, int* shifts, cudaStream_t st);

// sum += |frames| shifted back by their shifts (Array2::shifted semantics);
// the stack's frame 0 enters with its sign (smip-cli/main.cpp:266).
cudaError_t launch_saa_add(int dtype, void* sum, const void* frames, long long frame_stride_elems, int nframes,
                           int first_is_frame0, const int* shifts, const Geometry& g, cudaStream_t st);

// Mixed-radix counterparts of the three launchers above for the generic path
// (k_fftg.cu); same inputs and outputs, twiddles from the stack's GenTw tables.
cudaError_t launch_gen_row_pass(int dtype, const void* frames, long long fstride, int nframes, const Geometry& g,
                                dfc* Gt, const dfc* twW, cudaStream_t st, void* copy_out = nullptr);
cudaError_t launch_gen_col_pass(int mode, const dfc* Gt, float2* S, const float2* Rbuf, float2* Rout, float2* T,
                                double* Ppart, int nframes, int fpc, int skip_xcorr_frame0, const Geometry& g,
                                const dfc* twH, const float2* twH32, cudaStream_t st);
cudaError_t launch_gen_xcorr_rows(const float2* T, float* corr, float* rowmax, int nframes, const Geometry& g,
                                  const float2* twW32, cudaStream_t st);
// In-place FP64 transforms of nlines lines of length p.L (element stride es,
// line stride ls); sign -1 forward, +1 inverse (unnormalised).
cudaError_t launch_gen_lines_d(double2* data, const GenPlan& p, int nlines, long long ls, long long es, int sign,
                               const double2* tw, cudaStream_t st);

// FFT-order complex<double> spectra -> S layout (float2).
cudaError_t launch_import_spectra(const double* spectra, int nframes, const Geometry& g, float2* S, cudaStream_t st);

// Bispectrum accumulation over a batch of spectra S[0..nframes).
struct BispecLaunch {
    const float2* S;     // [nframes][hw][H]
    int nframes;
    float2* B;           // packed bispectrum
    float2* C;           // Kahan compensation, same layout
    int* err;
    int num_sms;
    float2* scratch;     // bispec_scratch_bytes(num_sms): partial sums of split tiles
    int* tile_cnt;       // bispec_tile_counters(num_sms) ints, zeroed once: parts finished per split tile
    int variant = 0;     // kernel staging: 0 four frames per ring stage, 1 two
    int min_part = 0;    // frames per split-tile part at least (0: 8)
};
cudaError_t launch_bispec_accumulate(const BispecLaunch& L, const Geometry& g, cudaStream_t st);
cudaError_t launch_bispec_accumulate_fps2(const BispecLaunch& L, const Geometry& g, cudaStream_t st);
size_t bispec_scratch_bytes(int num_sms);

// Many stacks' batches in one persistent launch (k_bispec.cu).  A record per
// stack (bispec_multi_rec_bytes() bytes, 64-byte aligned) holds its tensor
// maps and launch arguments; bispec_multi_fill writes it for the batch L and
// returns the stack's unit count (tiles and split-tile parts, as its own
// launch would run them) with each unit's frames, or -1.  The launch takes
// units from items[0 .. ctrl[0]) = (record, unit), counting ctrl[1] up from
// zero; records, items and ctrl are device memory.
size_t bispec_multi_rec_bytes();
int bispec_multi_fill(void* rec, const BispecLaunch& L, const Geometry& g, std::vector<int>* unit_frames);
cudaError_t launch_bispec_multi(const void* recs, const int2* items, int* ctrl, int num_sms, cudaStream_t st);
// diagnostic: two bounded waits that can never be satisfied (see smip_diag_bounded_wait)
cudaError_t launch_bounded_wait_probe(int* err, const int* never, double timeout_s, cudaStream_t st);
size_t bispec_tile_counters(int num_sms);
bool bispec_depth_supported(int De);

// out = (B - C) / nframes  (float2 packed), or plain add dst += src for merge.
cudaError_t launch_bispec_normalize(const float2* B, const float2* C, double nframes, long long n, float2* out,
                                    cudaStream_t st);
cudaError_t launch_bispec_merge(float2* Bd, float2* Cd, const float2* Bs, const float2* Cs, long long n,
                                cudaStream_t st);

// Closure-phase recovery (one CTA per job).
struct RecoJob {
    const float2* B;     // normalised packed bispectrum
    const int2* visits;  // spiral visit list
    int nvisits;
    int W, H, De;
    double2* phases;     // W*H, FFT order
    float2* phf;         // FP32 phases used along the chain (scratch)
    float2* plan;        // [nvisits][(De+1)^2] unit phasors of B for every (visit, v)
    float4* sums;        // per point: float-float phasor sums (re hi, re lo, im hi, im lo)
    int* cnt;            // per point: number of phasors (-1 for the seeds)
    double* cons;        // W*H
    unsigned char* flags;
    int* err;
    // pipelined walk: per point its first three visit indices and its visit
    // count (-1 padded); per visit the pairs whose u or v was visited within
    // the last kRecoLag visits (bitmask over the (De+1)^2 pair slots), and
    // their slots as a list (count -1: more than kRecentMax)
    const int4* pvis;
    unsigned* rbits;
    int* rcount;
    unsigned short* rlist;
};
constexpr int kRecoLag = 32;     // visits between a point's phase and the parallel stage's use of it
constexpr int kRecentMax = 64;   // recent pairs per visit the serial warp takes from a list
cudaError_t launch_phase_reco(const RecoJob* jobs_dev, int njobs, int max_W, int max_H, int max_De, cudaStream_t st);
// Ring-parallel estimator (opt-in, not the reference's): rq holds the spiral's
// visit indices grouped by ring, ring k at [roff[k], roff[k+1]); fring: W*H ints.
cudaError_t launch_ring_reco(const RecoJob* job_dev, int* fring, const int* rq, const std::vector<int>& roff, int W,
                             int H, cudaStream_t st);
// get_element index replica over a list of (ux, uy, vx, vy) tuples
cudaError_t launch_offset_probe(const Geometry& g, const int* idx, long long n, long long* off, int* conj,
                                cudaStream_t st);

// Final image (double precision): Z = sqrt(P_norm) * (phases * hann), inverse
// FFT, divide by max |.|.  Also writes the full-plane normalised power.
cudaError_t launch_finish(const double* Phalf, double pnorm, const double2* phases, double aperture,
                          const Geometry& g, double2* Z, double* power_full, double* maxbuf, const double2* tw64,
                          cudaStream_t st,
                          const double2* twW64 = nullptr, const double2* twH64 = nullptr);
cudaError_t launch_power_full(const double* Phalf, double pnorm, const Geometry& g, double* power_full,
                              cudaStream_t st);
cudaError_t launch_hann(double* out, int W, int H, double aperture, cudaStream_t st);
// Array2<double>::shifted: out(x, y) = in(x - dx, y - dy), zero outside.
cudaError_t launch_shifted(const double* in, double* out, int W, int H, int dx, int dy, cudaStream_t st);

// Sum of squares of a frame (double), for the correlation error bound.
cudaError_t launch_sumsq(int dtype, const void* frame, long long n, double* out, cudaStream_t st);

} // namespace smip_gpu
