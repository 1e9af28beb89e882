// C++ layer check: the reference's call pattern through smip::gpu (include/
// smip/gpu.hpp).  Writes results as raw little-endian files into argv[1] for
// the Python test to compare with the ctypes binding.
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <random>
#include <string>

#include "smip/gpu.hpp"

template <class T> static void dump(const std::string& path, const T* p, std::size_t n)
{
    std::ofstream(path, std::ios::binary).write(reinterpret_cast<const char*>(p), sizeof(T) * n);
}

int main(int argc, char** argv)
{
    if (argc != 2)
        return 2;
    const std::string dir = argv[1];
    namespace g = smip::gpu;
    const std::size_t N = 64;
    // frames: seeded integers, as Array2-like images
    std::mt19937 rng(5);
    std::vector<g::Image<double>> frames;
    for (int f = 0; f < 6; ++f) {
        g::Image<double> im(N, N);
        for (auto& v : im)
            v = (double)(rng() % 4096);
        frames.push_back(im);
    }
    // CrossCorrelation<double>: get_displacement before correlate throws bad_function_call
    g::CrossCorrelation<double> xc(frames[0]);
    bool threw = false;
    try {
        (void)xc.get_displacement();
    } catch (const std::bad_function_call&) {
        threw = true;
    }
    if (!threw)
        return 3;
    const auto sh = xc(frames[1]);
    const int shv[2] = { sh[0], sh[1] };
    dump(dir + "/xc_shift.bin", shv, 2);
    // Stack: the smip-cli pipeline
    g::Stack st(N, N, 20);
    for (const auto& fr : frames)
        st.push_frame(fr);
    const auto b = st.bispectrum();
    dump(dir + "/stack_bispec.bin", b.data(), b.size());
    g::PhaseMap pm;
    const auto ph = st.reconstruct_phases(24.0, &pm);
    dump(dir + "/stack_phases.bin", ph.data(), ph.size());
    dump(dir + "/stack_flags.bin", pm.flag.data(), pm.flag.size());
    // Bispectrum + reconstruct_phases free function; write/read round trip
    g::Bispectrum bs({ N, N, 20, 20 });
    g::Image<std::complex<double>> spec(N, N);
    for (std::size_t i = 0; i < spec.size(); ++i)
        spec.data()[i] = { (double)(i % 97), (double)(i % 31) - 15.0 };
    bs.accumulate_from_fft(spec);
    bs.write_to_file(dir + "/b.dat");
    g::Bispectrum bs2({ N, N, 20, 20 });
    bs2.read_from_file(dir + "/b.dat");
    const auto p1 = g::reconstruct_phases(bs, N, N, 24.0);
    const auto p2 = g::reconstruct_phases(bs2, N, N, 24.0);
    for (std::size_t i = 0; i < p1.size(); ++i)
        if (p1.data()[i] != p2.data()[i])
            return 4;
    // whole-stack checkpoint: 3 frames, save, load into a new stack, 3 more
    // frames -> the bispectrum of one stack that takes all 6 (3-frame
    // batches, so that both sum the same frames per batch)
    {
        g::Stack u(N, N, 20, 0, nullptr, 3);
        for (int f = 0; f < 6; ++f)
            u.push_frame(frames[f]);
        g::Stack a(N, N, 20, 0, nullptr, 3);
        for (int f = 0; f < 3; ++f)
            a.push_frame(frames[f]);
        a.save_state(dir + "/state.bin");
        g::Stack c(N, N, 20, 0, nullptr, 3);
        c.load_state(dir + "/state.bin");
        for (int f = 3; f < 6; ++f)
            c.push_frame(frames[f]);
        if (c.bispectrum() != u.bispectrum())
            return 7;
        // the bispectrum from memory reconstructs as the original stack does
        g::Stack m(N, N, 20);
        m.set_bispectrum(b); // nframes 1: the accumulator holds b itself
        const auto phm = m.reconstruct_phases(24.0);
        if (!std::equal(phm.begin(), phm.end(), ph.begin()))
            return 8;
        // frame-level sharding: src shares the reference, then merges
        g::Stack d0(N, N, 20), d1(N, N, 20);
        d0.push_frame(frames[0]);
        d0.share_reference(d1);
        for (int f = 1; f < 6; ++f)
            (f < 3 ? d0 : d1).push_frame(frames[f]);
        d0.merge(d1);
        if (d0.nframes() != 6)
            return 9;
    }
    // errors map to the reference's exception types
    try {
        g::Hann<double>(N, N, 0.0);
        return 5;
    } catch (const std::domain_error&) {
    }
    try {
        g::Stack bad(2048, 64, 16); // frame sides above 1024 are refused
        return 6;
    } catch (const g::unsupported&) {
    }
    double r = 0, phi = 0;
    int i = 0, j = 0;
    g::NextRecoIndex(r, phi, i, j);
    const int rij[2] = { i, j };
    dump(dir + "/next_reco.bin", rij, 2);
    const auto shf = g::shifted(frames[0], { 3, -2 });
    dump(dir + "/shifted.bin", shf.data(), shf.size());
    const auto w = g::Hann<double>(N, N, 48.0);
    dump(dir + "/hann.bin", w.data(), w.size());
    std::cout << "ok\n";
    return 0;
}
