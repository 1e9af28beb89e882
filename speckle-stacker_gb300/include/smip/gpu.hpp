// gpu.hpp -- C++ host layer of the GB300 SMIP engine (header only).
//
// The names and argument meanings follow hangeza/speckle-stacker v0.3.2's hot
// path API so that C++ callers switch by changing a namespace:
//
//   reference (namespace smip)                         here (namespace smip::gpu)
//   Bispectrum<complex<float>>({nx, ny, d, d})          Bispectrum({nx, ny, d, d})
//     .accumulate_from_fft(fft)  bispectrum.h:82-83       .accumulate_from_fft(fft)
//     .write_to_file / read_from_file  :56-60             .write_to_file / read_from_file
//   reconstruct_phases<T, U>(b, nx, ny, R, &pm)         reconstruct_phases(b, nx, ny, R, &pm)
//                                   phasereco.h:16-19
//   NextRecoIndex(r, phi, i, j)      phasereco.h:21     NextRecoIndex(r, phi, i, j)
//   CrossCorrelation<T>(ref), operator()(frame),        CrossCorrelation<T>(ref), operator()(frame),
//     get_displacement(), get_correlation_array()         get_displacement(), get_correlation_array()
//                                   crosscorrel.h:47-58
//   Hann<T>(nx, ny, aperture)  window_function.h:39-46  Hann<T>(nx, ny, aperture)
//   smip-cli/main.cpp:246-376 (the per-frame loop       Stack: push_frames, shifts, sum, power,
//     and the finish)                                    bispectrum, finish
//
// Inputs are any 2-D array with ncols(), nrows() and data() (a raw pointer or
// the reference's shared_ptr<T[]>), row-major with x fastest -- the
// reference's own Array2 works unchanged -- or a pointer plus sizes.  Results
// come back in Image<T>, which has the same accessors.  Every call goes
// through the C ABI of libsmip_gpu.so (include/smip_gpu.h); status codes turn
// into the exception types the reference throws:
//   SMIP_E_INVALID_ARGUMENT -> std::invalid_argument   SMIP_E_OUT_OF_RANGE -> std::out_of_range
//   SMIP_E_RUNTIME          -> std::runtime_error      SMIP_E_DOMAIN       -> std::domain_error
//   SMIP_E_BAD_CALL         -> std::bad_function_call  SMIP_E_NO_MEMORY    -> std::bad_alloc
//   SMIP_E_UNSUPPORTED      -> smip::gpu::unsupported (a std::invalid_argument)
//   SMIP_E_CUDA, SMIP_E_TIMEOUT -> smip::gpu::device_error (a std::runtime_error)
#pragma once

#include <array>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "smip_gpu.h"

namespace smip::gpu {

struct unsupported : std::invalid_argument {
    using std::invalid_argument::invalid_argument;
};
struct device_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void check(int rc)
{
    if (rc == SMIP_OK)
        return;
    const std::string msg = smip_last_error();
    switch (rc) {
    case SMIP_E_INVALID_ARGUMENT: throw std::invalid_argument(msg);
    case SMIP_E_OUT_OF_RANGE: throw std::out_of_range(msg);
    case SMIP_E_RUNTIME: throw std::runtime_error(msg);
    case SMIP_E_DOMAIN: throw std::domain_error(msg);
    case SMIP_E_BAD_CALL: throw std::bad_function_call();
    case SMIP_E_NO_MEMORY: throw std::bad_alloc();
    case SMIP_E_UNSUPPORTED: throw unsupported(msg);
    default: throw device_error(msg);
    }
}

namespace detail {
template <class P> auto raw(const P& p)
{
    if constexpr (std::is_pointer_v<P>)
        return p;
    else
        return p.get();
}
template <class A> auto data_of(const A& a) { return raw(a.data()); }
} // namespace detail

// Row-major 2-D host array (x fastest), the result type of this layer.
template <class T> class Image {
public:
    Image() = default;
    Image(std::size_t ncols, std::size_t nrows) : m_nx(ncols), m_ny(nrows), m_v(ncols * nrows) {}
    std::size_t ncols() const noexcept { return m_nx; }
    std::size_t nrows() const noexcept { return m_ny; }
    std::size_t size() const noexcept { return m_v.size(); }
    T* data() noexcept { return m_v.data(); }
    const T* data() const noexcept { return m_v.data(); }
    T& operator()(std::size_t x, std::size_t y) { return m_v[y * m_nx + x]; }
    const T& operator()(std::size_t x, std::size_t y) const { return m_v[y * m_nx + x]; }
    auto begin() noexcept { return m_v.begin(); }
    auto end() noexcept { return m_v.end(); }
    auto begin() const noexcept { return m_v.begin(); }
    auto end() const noexcept { return m_v.end(); }

private:
    std::size_t m_nx = 0, m_ny = 0;
    std::vector<T> m_v;
};

// PhaseMap (phasemap.h:10-20): per frequency a flag and a consistency value.
struct PhaseMap {
    Image<unsigned char> flag;
    Image<double> consistency;
};

// Frame element type of a C++ type, for push_frames.
template <class T> constexpr int dtype_of()
{
    if constexpr (std::is_same_v<T, std::uint8_t>)
        return SMIP_U8;
    else if constexpr (std::is_same_v<T, std::uint16_t>)
        return SMIP_U16;
    else if constexpr (std::is_same_v<T, float>)
        return SMIP_F32;
    else {
        static_assert(std::is_same_v<T, double>, "frames are uint8, uint16, float or double");
        return SMIP_F64;
    }
}

// ----------------------------------------------------------------- Stack
// One speckle-masking job: the accumulators of smip-cli/main.cpp:232-312 on
// the GPU (packed bispectrum + Kahan compensation, power spectrum, shift-and-
// add sum, reference frame, frame count).
class Stack {
public:
    Stack(std::size_t ncols, std::size_t nrows, std::size_t bdepth, int device = 0, void* stream = nullptr,
          long batch_frames = 0)
        : m_nx(ncols), m_ny(nrows), m_d(bdepth)
    {
        smip_stack_t h = nullptr;
        check(smip_stack_create(&h, device, (long)ncols, (long)nrows, (long)bdepth, stream, batch_frames));
        m_h.reset(h);
    }
    std::size_t ncols() const noexcept { return m_nx; }
    std::size_t nrows() const noexcept { return m_ny; }
    std::size_t bdepth() const noexcept { return m_d; }
    smip_stack_t handle() const noexcept { return m_h.get(); }

    // frames: count consecutive ncols x nrows frames (host or device memory)
    template <class T> void push_frames(const T* frames, std::size_t count, bool on_device = false)
    {
        check(smip_stack_push_frames(handle(), frames, dtype_of<T>(), (long)count, 0, on_device ? 1 : 0));
    }
    // one frame as a 2-D array (the reference's Array2<double> included)
    template <class A> void push_frame(const A& frame)
    {
        using T = std::remove_cv_t<std::remove_pointer_t<decltype(detail::data_of(frame))>>;
        check_shape(frame.ncols(), frame.nrows());
        push_frames<T>(detail::data_of(frame), 1);
    }
    // Bispectrum::accumulate_from_fft for spectra computed elsewhere
    void accumulate_fft(const std::complex<double>* spectra, std::size_t count, bool on_device = false)
    {
        check(smip_stack_accumulate_fft(handle(), reinterpret_cast<const double*>(spectra), (long)count,
                                        on_device ? 1 : 0));
    }
    void flush() { check(smip_stack_flush(handle())); }
    void sync() { check(smip_stack_sync(handle())); }
    void reset() { check(smip_stack_reset(handle())); }
    // SMIP_RECO_SPIRAL (the reference's walk, default) or SMIP_RECO_RINGS (ring-parallel, not the reference's)
    void set_reco_mode(int mode) { check(smip_stack_set_reco_mode(handle(), mode)); }
    long nframes() const
    {
        long n = 0;
        check(smip_stack_frame_count(handle(), &n));
        return n;
    }
    std::size_t bispectrum_size() const
    {
        long n = 0;
        check(smip_stack_bispectrum_size(handle(), &n));
        return (std::size_t)n;
    }
    // (x, y) shift of every frame against frame 0 (crosscorrel.h:166-179)
    std::vector<std::array<int, 2>> shifts() const
    {
        const long n = nframes();
        std::vector<std::array<int, 2>> v((std::size_t)n);
        if (n)
            check(smip_stack_shifts(handle(), v[0].data(), 0, n));
        return v;
    }
    Image<double> sum() const // sumarray / nframes (main.cpp:308)
    {
        Image<double> s(m_nx, m_ny);
        check(smip_stack_sum(handle(), s.data()));
        return s;
    }
    Image<double> power() const // powerspec / (nframes * size) (main.cpp:310)
    {
        Image<double> p(m_nx, m_ny);
        check(smip_stack_power(handle(), p.data()));
        return p;
    }
    std::vector<std::complex<float>> bispectrum() const // bispectrum / nframes (main.cpp:312)
    {
        std::vector<std::complex<float>> b(bispectrum_size());
        check(smip_stack_bispectrum(handle(), reinterpret_cast<float*>(b.data())));
        return b;
    }
    Image<std::complex<double>> reconstruct_phases(double reco_radius, PhaseMap* pm = nullptr) const
    {
        Image<std::complex<double>> ph(m_nx, m_ny);
        prepare(pm);
        check(smip_stack_reconstruct(handle(), reco_radius, reinterpret_cast<double*>(ph.data()),
                                     pm ? pm->flag.data() : nullptr, pm ? pm->consistency.data() : nullptr));
        return ph;
    }
    // main.cpp:318-376: phases, Hann window of aperture 2R, sqrt(P) x phases,
    // backward FFT, division by the largest modulus
    struct Result {
        Image<std::complex<double>> image, phases;
        PhaseMap pm;
    };
    Result finish(double reco_radius) const
    {
        Result r { Image<std::complex<double>>(m_nx, m_ny), Image<std::complex<double>>(m_nx, m_ny), {} };
        prepare(&r.pm);
        check(smip_stack_finish(handle(), reco_radius, reinterpret_cast<double*>(r.image.data()),
                                reinterpret_cast<double*>(r.phases.data()), r.pm.flag.data(),
                                r.pm.consistency.data()));
        return r;
    }
    // buffers and visit tables of finish(reco_radius) ahead of the first call
    void prepare_reco(double reco_radius) const { check(smip_stack_prepare_reco(handle(), reco_radius)); }
    void write_to_file(const std::string& path) const { check(smip_stack_save_bispectrum(handle(), path.c_str())); }
    void read_from_file(const std::string& path, long nframes = 0)
    {
        check(smip_stack_load_bispectrum(handle(), path.c_str(), nframes));
    }
    void merge(const Stack& src) { check(smip_stack_merge(handle(), src.handle())); }
    // src correlates against this stack's reference frame (before src's first frame; then merge(src))
    void share_reference(Stack& src) const { check(smip_stack_share_reference(handle(), src.handle())); }
    // the bispectrum.dat payload from memory (base_size normalised elements) into an empty stack
    void set_bispectrum(const std::vector<std::complex<float>>& b, long nframes = 0)
    {
        check(smip_stack_set_bispectrum(handle(), reinterpret_cast<const float*>(b.data()), nframes));
    }
    // whole-stack checkpoint: every accumulator, the frame count, shifts and reference frame
    void save_state(const std::string& path) const { check(smip_stack_save_state(handle(), path.c_str())); }
    void load_state(const std::string& path) { check(smip_stack_load_state(handle(), path.c_str())); }

protected:
    void check_shape(std::size_t nx, std::size_t ny) const
    {
        if (nx != m_nx || ny != m_ny)
            throw std::invalid_argument("frame dimensions differ from the stack's");
    }
    void prepare(PhaseMap* pm) const
    {
        if (pm) {
            pm->flag = Image<unsigned char>(m_nx, m_ny);
            pm->consistency = Image<double>(m_nx, m_ny);
        }
    }

private:
    struct Del {
        void operator()(smip_stack_t h) const noexcept { smip_stack_destroy(h); }
    };
    std::size_t m_nx, m_ny, m_d;
    std::unique_ptr<std::remove_pointer_t<smip_stack_t>, Del> m_h;
};

// ------------------------------------------------------------- Bispectrum
// Bispectrum<complex<float>> with device-resident storage: dims {ncols,
// nrows, bdepth, bdepth} as in bispectrum.h:183-192.
class Bispectrum : public Stack {
public:
    explicit Bispectrum(const std::array<std::size_t, 4>& dims, int device = 0, void* stream = nullptr)
        : Stack(dims[0], dims[1], dims[2], device, stream)
    {
        if (dims[3] != dims[2])
            throw std::invalid_argument("Bispectrum: dims 3 and 4 must be equal");
    }
    // FFT-order complex<double> spectrum of one frame (main.cpp:273, 298)
    template <class A> void accumulate_from_fft(const A& fft)
    {
        check_shape(fft.ncols(), fft.nrows());
        accumulate_fft(reinterpret_cast<const std::complex<double>*>(detail::data_of(fft)), 1);
    }
    std::size_t size() const { return bispectrum_size(); }
    std::size_t base_size() const { return bispectrum_size(); }
};

// reconstruct_phases<complex_t, complex<float>>(bispectrum, xsize, ysize, R, &pm)
inline Image<std::complex<double>> reconstruct_phases(const Bispectrum& b, std::size_t xsize, std::size_t ysize,
                                                      double reco_radius, PhaseMap* pm = nullptr)
{
    if (xsize != b.ncols() || ysize != b.nrows())
        throw std::invalid_argument("reconstruct_phases: size differs from the bispectrum's");
    return b.reconstruct_phases(reco_radius, pm);
}

// reconstruct_phases on a host packed bispectrum (complex<float>, base_size)
inline Image<std::complex<double>> reconstruct_phases(const std::complex<float>* bispec, std::size_t xsize,
                                                      std::size_t ysize, std::size_t bdepth, double reco_radius,
                                                      PhaseMap* pm = nullptr, int device = 0)
{
    Image<std::complex<double>> ph(xsize, ysize);
    if (pm) {
        pm->flag = Image<unsigned char>(xsize, ysize);
        pm->consistency = Image<double>(xsize, ysize);
    }
    check(smip_reconstruct_phases(device, reinterpret_cast<const float*>(bispec), (long)xsize, (long)ysize,
                                  (long)bdepth, reco_radius, reinterpret_cast<double*>(ph.data()),
                                  pm ? pm->flag.data() : nullptr, pm ? pm->consistency.data() : nullptr));
    return ph;
}

inline void NextRecoIndex(double& r, double& phi, int& i, int& j) { check(smip_next_reco_index(&r, &phi, &i, &j)); }

// --------------------------------------------------------- CrossCorrelation
// CrossCorrelation<T> (crosscorrel.h:47-58): shift of a frame against the
// reference frame given at construction, first maximum in row-major order,
// wrapped to a signed shift.
template <class T = double> class CrossCorrelation {
public:
    template <class A> explicit CrossCorrelation(const A& ref, int device = 0) : m_dev(device)
    {
        m_nx = ref.ncols();
        m_ny = ref.nrows();
        m_ref = to_double(detail::data_of(ref), m_nx * m_ny);
    }
    template <class A> void correlate(const A& frame)
    {
        if (frame.ncols() != m_nx || frame.nrows() != m_ny)
            throw std::invalid_argument("CrossCorrelation: frame dimensions differ from the reference's");
        const std::vector<double> f = to_double(detail::data_of(frame), m_nx * m_ny);
        m_corr = Image<double>(m_nx, m_ny);
        check(smip_xcorr_displacement(m_dev, m_ref.data(), f.data(), (long)m_nx, (long)m_ny, &m_shift[0],
                                      &m_shift[1], m_corr.data()));
        m_ready = true;
    }
    template <class A> std::array<int, 2> operator()(const A& frame)
    {
        correlate(frame);
        return m_shift;
    }
    std::array<int, 2> get_displacement() const
    {
        if (!m_ready)
            throw std::bad_function_call(); // crosscorrel.h:155-159
        return m_shift;
    }
    const Image<double>& get_correlation_array() const
    {
        if (!m_ready)
            throw std::bad_function_call(); // crosscorrel.h:147-152
        return m_corr;
    }
    template <class A, class B> static std::array<int, 2> get_displacement(const A& a, const B& b)
    {
        CrossCorrelation<T> c(a);
        return c(b);
    }

private:
    template <class U> static std::vector<double> to_double(const U* p, std::size_t n)
    {
        std::vector<double> v(n);
        for (std::size_t i = 0; i < n; ++i) {
            if constexpr (std::is_arithmetic_v<U>)
                v[i] = (double)p[i];
            else
                v[i] = std::abs(p[i]); // complex frames: modulus, as main.cpp:289 passes them
        }
        return v;
    }
    int m_dev;
    std::size_t m_nx = 0, m_ny = 0;
    std::vector<double> m_ref;
    Image<double> m_corr;
    std::array<int, 2> m_shift { 0, 0 };
    bool m_ready = false;
};

// Array2<T>::shifted(distance) (array2.h:603-622), on the GPU in double:
// element (x, y) of the result is a(x - dx, y - dy), zero outside.
template <class T> Image<double> shifted(const Image<T>& a, std::array<int, 2> distance, int device = 0)
{
    std::vector<double> in(a.begin(), a.end());
    Image<double> out(a.ncols(), a.nrows());
    check(smip_shifted(device, in.data(), out.data(), (long)a.ncols(), (long)a.nrows(), distance[0], distance[1]));
    return out;
}

// Hann<T>(xsize, ysize, aperture) (window_function.h:39-46, 70-85)
template <class T = double> Image<T> Hann(std::size_t xsize, std::size_t ysize, double aperture, int device = 0)
{
    Image<double> w(xsize, ysize);
    check(smip_hann(device, w.data(), (long)xsize, (long)ysize, aperture));
    if constexpr (std::is_same_v<T, double>)
        return w;
    else {
        Image<T> r(xsize, ysize);
        for (std::size_t i = 0; i < w.size(); ++i)
            r.data()[i] = T(w.data()[i]);
        return r;
    }
}

} // namespace smip::gpu
