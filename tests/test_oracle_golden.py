"""The CPU oracle against fixtures produced by the reference's own code
(tests/golden/make_golden.py) and against the reference's unit-test checks
(tests/bispectrum_test.cpp, tests/correl_test.cpp)."""
import numpy as np
import pytest
from conftest import golden

from oracle import bispec_desc


@pytest.mark.parametrize("name", ["stack_binary32_u8", "stack_ext64_u16"])
def test_oracle_pipeline_bit_exact(oracle, name):
    """smip-cli/main.cpp:246-378 restated: every output bit-identical to the
    reference compiled without fast-math."""
    fx = golden(name)
    out = oracle.run_stack(fx["frames"], int(fx["bdepth"]), float(fx["reco_radius"]))
    assert np.array_equal(out["shifts"], fx["shifts"])
    assert np.array_equal(out["shifts"], fx["shifts_fast"])
    assert np.array_equal(out["sum"].view(np.uint64), fx["sum"].view(np.uint64))
    assert np.array_equal(out["power"].real.view(np.uint64), fx["power"].view(np.uint64))
    assert np.array_equal(out["flags"], fx["flags"])
    assert np.array_equal(out["phases"].view(np.uint64), fx["phases"].view(np.uint64))
    assert np.array_equal(out["consistency"].view(np.uint64), fx["consistency"].view(np.uint64))
    assert np.array_equal(out["image"].view(np.uint64), fx["image"].view(np.uint64))
    b = out["bispec"]
    assert np.array_equal(b[fx["bispec_sample_idx"]].view(np.uint32), fx["bispec_sample"].view(np.uint32))
    if "bispec" in fx:
        assert np.array_equal(b.view(np.uint32), fx["bispec"].view(np.uint32))


def test_descriptor_table():
    """bispectrum.h:143-160, 203-220 incl. ConstructionTest (bispectrum_test.cpp:33-41)."""
    fx = golden("bispec_index")
    for row in fx["describe"]:
        nc, nr, d = (int(x) for x in row[:3])
        got = bispec_desc(nc, nr, d)
        exp = list(row[3:])
        assert got["sizes"] + got["base_sizes"] + [got["base_size"], got["totalsize"]] + got["min"] + got["max"] == exp
    c = bispec_desc(2, 3, 4)  # extents {2,3,4,5} in the reference test: sizes {3,3,5,5}
    assert c["sizes"][:2] == [3, 3] and c["sizes"][2] == 5


@pytest.mark.parametrize("key", ["n16_d4", "n24_d6", "n32_d8"])
def test_get_element_offsets(oracle, key):
    """Bispectrum::get_element index path, every pair calc_phase can query."""
    fx = golden("bispec_index")
    n, d = (int(x[1:]) for x in key.split("_"))
    off, cj = oracle.get_element_offsets(n, n, d, fx[key + "_idx"])
    assert np.array_equal(off, fx[key + "_off"])
    assert np.array_equal(cj, fx[key + "_conj"])


def test_element_access_round_trip(oracle):
    """ElementAccess (bispectrum_test.cpp:51-61): calc_indices then get_element
    returns the element itself for every packed offset."""
    import ctypes as C
    for (nc, nr, d) in [(3, 4, 5), (8, 8, 4), (16, 8, 6)]:
        desc = (C.c_long * 24)()
        oracle.lib.orc_bispec_describe(C.c_long(nc), C.c_long(nr), C.c_long(d), C.c_long(d), desc)
        bs = bispec_desc(nc, nr, d)["base_size"]
        idx = np.zeros((bs, 4), np.int32)
        buf = (C.c_int * 4)()
        for a in range(bs):
            oracle.lib.orc_calc_indices(desc, C.c_long(a), buf)
            idx[a] = list(buf)
        off, cj = oracle.get_element_offsets(nc, nr, d, idx)
        assert np.array_equal(off, np.arange(bs))
        assert not cj.any()


def test_complex_conjugation(oracle):
    """ComplexConjugation (bispectrum_test.cpp:67-70): B(1,-2,1,-1) = conj B(-1,2,-1,1)."""
    o1, c1 = oracle.get_element_offsets(4, 4, 4, np.array([[-1, 2, -1, 1], [1, -2, 1, -1]], np.int32))
    assert o1[0] == o1[1] and c1[0] == 0 and c1[1] == 1


def test_zero_size_throws(oracle):
    """ZeroSize (bispectrum_test.cpp:73-79): get_element on an empty bispectrum throws."""
    import ctypes as C
    desc = (C.c_long * 24)()  # default-constructed: every size and base_size zero
    idx = (C.c_int * 4)(0, 0, 0, 0)
    cj = C.c_int()
    assert oracle.lib.orc_get_element_offset(desc, idx, C.byref(cj)) == -1


def test_reco_visits(oracle):
    fx = golden("reco_visits")
    import hashlib
    for R in (12, 24, 32, 64, 128, 200):
        v = oracle.reco_visits(R)
        assert len(v) == int(fx[f"r{R}_count"])
        assert hashlib.sha256(v.astype(np.int32).tobytes()).hexdigest() == str(fx[f"r{R}_sha"])
        if f"r{R}" in fx:
            assert np.array_equal(v, fx[f"r{R}"])


def test_xcorr_gaussian(oracle):
    """correl_test.cpp restated with a seed: the measured shifts equal the
    generated integer shifts and the reference's own measurements."""
    fx = golden("xcorr_gauss")
    g = fx["gaus"]
    for (dx, dy), m in zip(fx["generated"], fx["measured"]):
        s = oracle.xcorr(g, oracle.shifted(g, int(dx), int(dy)))
        assert s == tuple(m) == (dx, dy)


def test_fft_against_numpy(oracle):
    rng = np.random.default_rng(3)
    for shape in [(16, 16), (32, 64), (12, 20)]:
        a = rng.normal(size=shape) + 1j * rng.normal(size=shape)
        got = oracle.fft2(a, -1)
        exp = np.fft.fft2(a)
        assert np.abs(got - exp).max() <= 1e-12 * np.abs(exp).max()
        assert np.abs(oracle.fft2(a, +1) - np.fft.ifft2(a) * a.size).max() <= 1e-12 * np.abs(exp).max()


def test_hann_and_shifted(oracle):
    w = oracle.hann(8, 8, 6.0)
    assert w[0, 0] == 1.0 and np.allclose(w, w.T)
    a = np.arange(16, dtype=float).reshape(4, 4)
    s = oracle.shifted(a, 1, -1)
    assert s[0, 1] == a[1, 0] and s[3, 0] == 0.0


def test_accumulate_threads_invariant(oracle):
    rng = np.random.default_rng(9)
    F = np.fft.fft2(rng.integers(0, 255, (32, 32)).astype(float))
    d = bispec_desc(32, 32, 8)
    a = np.zeros(d["base_size"], np.complex64)
    b = a.copy()
    oracle.accumulate(a, F, 8, nthreads=1)
    oracle.accumulate(b, F, 8, nthreads=5)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_map_to_color_known_values(oracle):
    """mapToColor<uint16_t> (videoio.h:178-206) at its band edges and inside
    each band, worked out from the formula in double arithmetic and truncated
    as static_cast<uint16_t> does: value -> (r, g, b)."""
    M = 65535
    cases = {
        -0.5: (0, 0, 0), 0.0: (0, 0, 0), 0.1: (0, 0, 26214),          # 65535 * 0.4 truncated
        0.25: (0, 0, M), 0.3: (0, 13106, 52428),                      # 4*0.3-1 = 0.19999.. -> 13106.99..
        0.5: (0, M, 0), 0.6: (26213, 39321, 0),                        # 4*0.6-2 = 0.39999.. -> 26213.99..
        0.75: (M, 0, 0), 0.9: (M, 0, 39321),                           # 4*0.9-3 = 0.60000..1 -> 39321.00..
        1.0: (M, 0, M), 7.0: (M, 0, M), float("nan"): (0, 0, 0),
    }
    v = np.array(list(cases.keys()))
    got = oracle.map_to_color(v)
    for k, (value, exp) in enumerate(cases.items()):
        assert tuple(int(x) for x in got[k]) == exp, (value, got[k], exp)


def test_array2mat_order(oracle):
    """Array2Mat with signed_symmetry shows element (x - n/2, y - n/2) at
    pixel (x, y): an fftshift for even sizes; the identity without it."""
    a = np.arange(6 * 8, dtype=float).reshape(6, 8)
    assert np.array_equal(oracle.array2mat_order(a, True), np.fft.fftshift(a))
    assert np.array_equal(oracle.array2mat_order(a, False), a)
    b = np.arange(5 * 7, dtype=float).reshape(5, 7)   # odd sizes: min index -(n/2)
    assert np.array_equal(oracle.array2mat_order(b, True), np.roll(b, (2, 3), axis=(0, 1)))
