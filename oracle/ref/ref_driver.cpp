// ref_driver.cpp -- extern "C" entry points over the REFERENCE's own headers
// (hangeza/speckle-stacker v0.3.2, compiled in place from its include/ and
// src/ directories by oracle/ref/Makefile).  TEST INFRASTRUCTURE: it lets the
// Python tests and tests/golden/make_golden.py run the reference's code on the
// same inputs as the plain-C oracle and the CUDA library.
//
// Nothing here re-implements the reference: every function constructs the
// reference's classes and calls its templates.  ref_run_stack restates the
// control flow of smip-cli/main.cpp:246-378 with frames taken from a buffer
// instead of OpenCV (OpenCV is not installed here).
#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <vector>

#include "array2.h"
#include "bispectrum.h"
#include "crosscorrel.h"
#include "phasemap.h"
#include "phasereco.h"
#include "types.h"
#include "window_function.h"

using namespace smip;

namespace {

Array2<complex_t> spectrum_from(const double* fft, long ncols, long nrows)
{
    Array2<complex_t> a(ncols, nrows);
    for (long n = 0; n < ncols * nrows; ++n)
        a.begin()[n] = complex_t(fft[2 * n], fft[2 * n + 1]);
    return a;
}

template <typename C>
Bispectrum<C> make_bispec(long ncols, long nrows, long depth)
{
    using E = typename Bispectrum<C>::extents;
    return Bispectrum<C>(E { std::size_t(ncols), std::size_t(nrows), std::size_t(depth), std::size_t(depth) });
}

double pixel(const void* frames, int dtype, long n)
{
    switch (dtype) {
    case 0: return double(static_cast<const std::uint8_t*>(frames)[n]);
    case 1: return double(static_cast<const std::uint16_t*>(frames)[n]);
    case 2: return double(static_cast<const float*>(frames)[n]);
    default: return static_cast<const double*>(frames)[n];
    }
}

} // namespace

extern "C" {

// sizes[4], base_sizes[4], base_size, totalsize, min[4], max[4] -> 18 longs
int ref_describe(long ncols, long nrows, long depth, long* out)
{
    auto b = make_bispec<std::complex<double>>(ncols, nrows, depth);
    for (int n = 0; n < 4; ++n) {
        out[n] = long(b.sizes()[n]);
        out[4 + n] = long(b.base_sizes()[n]);
        out[10 + n] = long(b.min_indices()[n]);
        out[14 + n] = long(b.max_indices()[n]);
    }
    out[8] = long(b.base_size());
    out[9] = long(b.totalsize());
    return 0;
}

int ref_accumulate_f32(float* B, const double* fft, long ncols, long nrows, long depth)
{
    auto b = make_bispec<std::complex<float>>(ncols, nrows, depth);
    std::memcpy(b.data().get(), B, sizeof(float) * 2 * b.base_size());
    b.accumulate_from_fft(spectrum_from(fft, ncols, nrows));
    std::memcpy(B, b.data().get(), sizeof(float) * 2 * b.base_size());
    return 0;
}

int ref_accumulate_f64(double* B, const double* fft, long ncols, long nrows, long depth)
{
    auto b = make_bispec<std::complex<double>>(ncols, nrows, depth);
    std::memcpy(b.data().get(), B, sizeof(double) * 2 * b.base_size());
    b.accumulate_from_fft(spectrum_from(fft, ncols, nrows));
    std::memcpy(B, b.data().get(), sizeof(double) * 2 * b.base_size());
    return 0;
}

// For each 4-index tuple, report which packed element get_element returns
// (and whether conjugated) by filling the array with unique values; -1 where
// get_element throws.
int ref_get_element_probe(long ncols, long nrows, long depth, const int* idx, long n,
                          long* out_off, int* out_conj)
{
    auto b = make_bispec<std::complex<double>>(ncols, nrows, depth);
    for (std::size_t a = 0; a < b.base_size(); ++a)
        b.data()[a] = std::complex<double>(double(a), 1.0);
    for (long q = 0; q < n; ++q) {
        try {
            auto v = b.get_element({ idx[4 * q], idx[4 * q + 1], idx[4 * q + 2], idx[4 * q + 3] });
            out_off[q] = long(v.real());
            out_conj[q] = v.imag() < 0 ? 1 : 0;
        } catch (const std::out_of_range&) {
            out_off[q] = -1;
            out_conj[q] = 0;
        }
    }
    return 0;
}

long ref_calc_offset(long ncols, long nrows, long depth, const int* idx4)
{
    auto b = make_bispec<std::complex<double>>(ncols, nrows, depth);
    return long(b.calc_offset({ idx4[0], idx4[1], idx4[2], idx4[3] }));
}

int ref_calc_indices(long ncols, long nrows, long depth, long addr, int* idx4)
{
    auto b = make_bispec<std::complex<double>>(ncols, nrows, depth);
    auto v = b.calc_indices(std::size_t(addr));
    for (int n = 0; n < 4; ++n)
        idx4[n] = v[n];
    return 0;
}

void ref_next_reco_index(double* r, double* phi, int* i, int* j)
{
    NextRecoIndex(*r, *phi, *i, *j);
}

static int reco_out(const Array2<complex_t>& ph, const PhaseMap& pm, long np,
                    double* phases, unsigned char* flags, double* cons)
{
    for (long n = 0; n < np; ++n) {
        phases[2 * n] = ph.begin()[n].real();
        phases[2 * n + 1] = ph.begin()[n].imag();
        flags[n] = pm.begin()[n].flag ? 1 : 0;
        if (cons)
            cons[n] = pm.begin()[n].consistency;
    }
    return 0;
}

int ref_reconstruct_phases_f32(const float* B, long xs, long ys, long depth, double R,
                               double* phases, unsigned char* flags, double* cons)
{
    auto b = make_bispec<std::complex<float>>(xs, ys, depth);
    std::memcpy(b.data().get(), B, sizeof(float) * 2 * b.base_size());
    try {
        PhaseMap pm;
        auto ph = reconstruct_phases<complex_t, std::complex<float>>(b, xs, ys, R, &pm);
        return reco_out(ph, pm, xs * ys, phases, flags, cons);
    } catch (const std::out_of_range&) {
        return -1;
    }
}

int ref_reconstruct_phases_f64(const double* B, long xs, long ys, long depth, double R,
                               double* phases, unsigned char* flags, double* cons)
{
    auto b = make_bispec<std::complex<double>>(xs, ys, depth);
    std::memcpy(b.data().get(), B, sizeof(double) * 2 * b.base_size());
    try {
        PhaseMap pm;
        auto ph = reconstruct_phases<complex_t, std::complex<double>>(b, xs, ys, R, &pm);
        return reco_out(ph, pm, xs * ys, phases, flags, cons);
    } catch (const std::out_of_range&) {
        return -1;
    }
}

int ref_xcorr(const double* ref, const double* frame, long ncols, long nrows, int* dx, int* dy, double* corr)
{
    Array2<double> a(ncols, nrows), f(ncols, nrows);
    std::memcpy(a.data().get(), ref, sizeof(double) * ncols * nrows);
    std::memcpy(f.data().get(), frame, sizeof(double) * ncols * nrows);
    CrossCorrelation<double> cc(a);
    auto s = cc(f);
    *dx = s[0];
    *dy = s[1];
    if (corr) {
        const auto& c = cc.get_correlation_array();
        std::memcpy(corr, c.data().get(), sizeof(double) * ncols * nrows);
    }
    return 0;
}

int ref_shifted(const double* in, double* out, long ncols, long nrows, int dx, int dy)
{
    Array2<double> a(ncols, nrows);
    std::memcpy(a.data().get(), in, sizeof(double) * ncols * nrows);
    auto s = a.shifted({ dx, dy });
    std::memcpy(out, s.data().get(), sizeof(double) * ncols * nrows);
    return 0;
}

int ref_hann(double* out, long xs, long ys, double aperture)
{
    try {
        Hann<double> w(xs, ys, aperture);
        std::memcpy(out, w.data().get(), sizeof(double) * xs * ys);
        return 0;
    } catch (const std::domain_error&) {
        return -1;
    }
}

int ref_bispec_write(const char* fn, const float* B, long ncols, long nrows, long depth)
{
    auto b = make_bispec<std::complex<float>>(ncols, nrows, depth);
    std::memcpy(b.data().get(), B, sizeof(float) * 2 * b.base_size());
    try {
        b.write_to_file(fn);
    } catch (const std::runtime_error&) {
        return -1;
    }
    return 0;
}

// Reads a bispectrum.dat; writes dims[4] and up to cap complex values.
long ref_bispec_read(const char* fn, float* B, long cap, long* dims)
{
    Bispectrum<std::complex<float>> b;
    try {
        b.read_from_file(fn);
    } catch (const std::runtime_error&) {
        return -1;
    }
    for (int n = 0; n < 4; ++n)
        dims[n] = long((b.sizes()[n] / 2) * 2); // sizes are (d/2)*2+1
    const long n = long(b.base_size());
    std::memcpy(B, b.data().get(), sizeof(float) * 2 * std::size_t(std::min(n, cap)));
    return n;
}

// smip-cli/main.cpp:246-378 without OpenCV; same output contract as
// orc_run_stack (oracle/smip_oracle.h).
int ref_run_stack(const void* frames, int dtype, long nframes, long ncols, long nrows,
                  long depth, double reco_radius, int fp64_bispec,
                  int* shifts, double* sumarray_out, double* powerspec_out,
                  float* bispec32_out, double* bispec64_out,
                  double* phases_out, unsigned char* flags_out, double* cons_out,
                  double* image_out)
{
    if (fp64_bispec)
        return -3; // the CLI only instantiates Bispectrum<complex<float>>
    const long np = ncols * nrows;
    auto load = [&](long f) {
        Array2<complex_t> a(ncols, nrows);
        for (long n = 0; n < np; ++n)
            a.begin()[n] = complex_t(pixel(frames, dtype, f * np + n), 0.);
        return a;
    };
    Array2<complex_t> powerspec;
    Array2<complex_t> indata;
    Bispectrum<bispec_complex_t> bispectrum;
    Array2<complex_t> phases;
    long cur = 0;
    indata = load(cur++);
    bispectrum = Bispectrum<bispec_complex_t>({ indata.ncols(), indata.nrows(), std::size_t(depth), std::size_t(depth) });
    fftw_plan forward_plan = fftw_plan_dft_2d(indata.nrows(), indata.ncols(),
        reinterpret_cast<fftw_complex*>(indata.data().get()),
        reinterpret_cast<fftw_complex*>(indata.data().get()),
        FFTW_FORWARD, FFTW_ESTIMATE);
    Array2<double> sumarray(indata.ncols(), indata.nrows());
    std::transform(indata.begin(), indata.end(), sumarray.begin(), [](const complex_t& c) { return c.real(); });
    CrossCorrelation<double> cross_correl(sumarray);
    if (shifts) {
        shifts[0] = 0;
        shifts[1] = 0;
    }
    fftw_execute(forward_plan);
    bispectrum.accumulate_from_fft(indata);
    std::transform(indata.begin(), indata.end(), indata.begin(),
        [](const complex_t& val) { return complex_t { std::norm(val), 0. }; });
    powerspec = indata;
    while (cur < nframes) {
        indata = complex_t {};
        indata += load(cur);
        auto xyshift = cross_correl(Array2<double>::convert<std::complex<double>>(indata, complex_abs<double>));
        if (shifts) {
            shifts[2 * cur] = xyshift[0];
            shifts[2 * cur + 1] = xyshift[1];
        }
        xyshift = -xyshift;
        sumarray += Array2<double>::convert<std::complex<double>>(indata, complex_abs<double>).shifted(xyshift);
        fftw_execute(forward_plan);
        bispectrum.accumulate_from_fft(indata);
        std::transform(indata.begin(), indata.end(), indata.begin(),
            [](const complex_t& val) { return complex_t { std::norm(val), 0. }; });
        powerspec += indata;
        ++cur;
    }
    const std::size_t nfr = std::size_t(nframes);
    sumarray /= nfr;
    powerspec /= nfr * powerspec.size();
    bispectrum /= bispec_complex_t(nfr, 0.);
    fftw_destroy_plan(forward_plan);
    if (sumarray_out)
        std::memcpy(sumarray_out, sumarray.data().get(), sizeof(double) * np);
    if (powerspec_out)
        std::memcpy(powerspec_out, powerspec.data().get(), sizeof(double) * 2 * np);
    if (bispec32_out)
        std::memcpy(bispec32_out, bispectrum.data().get(), sizeof(float) * 2 * bispectrum.base_size());
    (void)bispec64_out;

    PhaseMap pm;
    try {
        phases = reconstruct_phases<complex_t, bispec_complex_t>(bispectrum, indata.ncols(), indata.nrows(), reco_radius, &pm);
    } catch (const std::out_of_range&) {
        return -1;
    }
    if (phases_out)
        reco_out(phases, pm, np, phases_out, flags_out ? flags_out : std::vector<unsigned char>(np).data(), cons_out);
    Hann<complex_t> window_f(powerspec.ncols(), powerspec.nrows(), reco_radius * 2);
    phases *= window_f;
    Array2<complex_t> result_image(powerspec.ncols(), powerspec.nrows());
    std::transform(powerspec.begin(), powerspec.end(), result_image.begin(),
        [](const complex_t& val) { return complex_t { std::sqrt(val.real()), 0. }; });
    result_image *= phases;
    fftw_plan reverse_plan = fftw_plan_dft_2d(result_image.nrows(), result_image.ncols(),
        reinterpret_cast<fftw_complex*>(result_image.data().get()),
        reinterpret_cast<fftw_complex*>(result_image.data().get()),
        FFTW_BACKWARD, FFTW_ESTIMATE);
    fftw_execute(reverse_plan);
    fftw_destroy_plan(reverse_plan);
    auto abscomp = [](const std::complex<double>& a, const std::complex<double>& b) {
        return (std::abs(a) < std::abs(b));
    };
    auto minmax = std::minmax_element(result_image.begin(), result_image.end(), abscomp);
    double normfact = std::abs(*(minmax.second));
    result_image /= complex_t { normfact, 0. };
    if (image_out)
        std::memcpy(image_out, result_image.data().get(), sizeof(double) * 2 * np);
    return 0;
}

} // extern "C"
