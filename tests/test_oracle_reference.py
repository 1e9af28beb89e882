"""The oracle against the reference's own code compiled in place
(oracle/_ref, built by `make -C oracle ref` where the reference sources are
present).  Randomised inputs beyond the committed fixtures."""
import numpy as np
import pytest

from oracle import Reference, bispec_desc

pytestmark = pytest.mark.skipif(not Reference.available("strict"), reason="reference build not present")


@pytest.fixture(scope="module")
def ref():
    return Reference("strict")


@pytest.mark.parametrize("shape", [(16, 16, 4), (32, 16, 8), (16, 32, 6), (24, 24, 10)])
def test_accumulate_bit_exact(oracle, ref, shape):
    nc, nr, d = shape
    rng = np.random.default_rng(nc * 100 + d)
    F = np.fft.fft2(rng.integers(0, 4000, (nr, nc)).astype(float))
    desc = bispec_desc(nc, nr, d)
    a = np.zeros(desc["base_size"], np.complex64)
    b = a.copy()
    for k in range(2):
        ref.accumulate(a, F * (k + 1), d)
        oracle.accumulate(b, F * (k + 1), d, nthreads=3)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("shape", [(16, 16, 4, 7), (32, 32, 8, 14), (32, 16, 6, 9)])
def test_reconstruct_bit_exact(oracle, ref, shape):
    nc, nr, d, R = shape
    rng = np.random.default_rng(R)
    desc = bispec_desc(nc, nr, d)
    B = np.zeros(desc["base_size"], np.complex64)
    for _ in range(3):
        oracle.accumulate(B, np.fft.fft2(rng.integers(0, 255, (nr, nc)).astype(float)), d)
    p1, f1, c1 = ref.reconstruct_phases(B, nc, nr, d, R)
    p2, f2, c2 = oracle.reconstruct_phases(B, nc, nr, d, R)
    assert np.array_equal(f1, f2)
    assert np.array_equal(p1.view(np.uint64), p2.view(np.uint64))
    assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64))


def test_get_element_rectangular(oracle, ref):
    idx = []
    for uy in range(-8, 8):
        for ux in range(-16, 16):
            for vy in range(-3, 4):
                for vx in range(-3, 4):
                    idx.append((ux, uy, vx, vy))
    idx = np.array(idx, np.int32)
    o1, c1 = ref.get_element_offsets(32, 16, 6, idx)
    o2, c2 = oracle.get_element_offsets(32, 16, 6, idx)
    assert np.array_equal(o1, o2) and np.array_equal(c1, c2)


def test_xcorr_random(oracle, ref):
    rng = np.random.default_rng(11)
    a = rng.integers(0, 255, (32, 32)).astype(float)
    for _ in range(10):
        b = np.roll(a, tuple(rng.integers(-16, 16, 2)), axis=(0, 1)) + rng.integers(0, 30, (32, 32))
        assert ref.xcorr(a, b) == oracle.xcorr(a, b)


def test_bispectrum_file_format(tmp_path, ref):
    """IO_Write_And_Read (bispectrum_test.cpp:132-149): size_t base_size,
    4 x size_t dims, then complex<float>[base_size]."""
    d = bispec_desc(8, 8, 4)
    B = (np.arange(d["base_size"]) + 1j).astype(np.complex64)
    fn = str(tmp_path / "b.dat")
    assert ref.write_bispec(fn, B, 8, 8, 4) == 0
    raw = open(fn, "rb").read()
    hdr = np.frombuffer(raw[:40], np.uint64)
    assert list(hdr) == [d["base_size"], 8, 8, 4, 4]
    assert np.array_equal(np.frombuffer(raw[40:], np.complex64), B)
