"""GPU parity for frame sizes that are not powers of two in [16, 512].

The reference takes frames of any size: FFTW plans whatever the frames have
(smip-cli/main.cpp:256-259, crosscorrel.h:112-141) and -s crops to any w:h
(main.cpp:157-167).  Such sizes run the mixed-radix transforms (k_fftg.cu),
and odd nrows change the packed bispectrum's u_y extent to nrows
((nrows/2)*2 + 1, bispectrum.h:203-220).  Against the FP64 oracle on the same
frames, with the tolerances of the power-of-two parity tests:

  shifts, shift-and-add sum, phase-map flags ............ bit-exact
  power spectrum ........ max |dP| <= 1e-6 max P
  bispectrum (normalised) rel-L2 <= 1e-5
  phases ................ max |dphi| <= 1e-3 rad, RMS <= 1e-4 rad (flagged points)
  image ................. rel-L2 <= 1e-4
"""
import numpy as np
import pytest
from conftest import phase_err, rel_l2

from oracle import bispec_desc

pytestmark = pytest.mark.gpu


def speckle_frames(W, H, n, dtype, seed):
    """A blob field, shifted by a few pixels per frame, with Poisson noise:
    every frame correlates with frame 0 at a distinct integer shift."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:H, 0:W].astype(float)
    base = np.zeros((H, W))
    for _ in range(12):
        x0, y0, s = rng.uniform(0.2 * W, 0.8 * W), rng.uniform(0.2 * H, 0.8 * H), rng.uniform(1.0, 3.0)
        base += rng.uniform(0.2, 1.0) * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * s * s))
    full = 200.0 if dtype == np.uint8 else 20000.0
    base = base / base.max() * full
    out = np.empty((n, H, W), dtype)
    for f in range(n):
        sh = (0, 0) if f == 0 else (int(rng.integers(-4, 5)), int(rng.integers(-4, 5)))
        img = np.roll(base, sh, axis=(0, 1)) + 0.03 * full
        out[f] = np.clip(rng.poisson(img), 0, np.iinfo(dtype).max).astype(dtype)
    return out


@pytest.mark.parametrize("W,H,D,R,n,dtype", [
    (96, 80, 16, 30, 10, np.uint16),     # 2^5 * 3 by 2^4 * 5
    (100, 100, 20, 40, 12, np.uint8),    # the reference's default depth
    (99, 75, 14, 28, 8, np.uint16),      # odd on both axes
    (37, 64, 8, 14, 6, np.uint16),       # a prime width
    (640, 480, 16, 60, 3, np.uint16),    # larger than 512
    (1024, 48, 8, 20, 3, np.uint16),     # a power of two above 512
])
def test_generic_size_pipeline(smip, oracle, W, H, D, R, n, dtype):
    frames = speckle_frames(W, H, n, dtype, seed=W * 31 + H)
    exp = oracle.run_stack(frames, D, float(R), fp64=True, nthreads=16)
    with smip.Stack(W, H, D, batch_frames=4) as st:  # several batches
        st.push_frames(frames)
        shifts, ssum, power, bispec = st.shifts(), st.sum(), st.power(), st.bispectrum()
        img, ph, fl, _ = st.finish(float(R))
    assert bispec.size == bispec_desc(W, H, D)["base_size"]
    assert np.array_equal(shifts, exp["shifts"])
    assert np.array_equal(ssum.view(np.uint64), np.asarray(exp["sum"]).view(np.uint64))
    p_exp = np.real(exp["power"])
    assert np.abs(power - p_exp).max() <= 1e-6 * p_exp.max()
    assert rel_l2(bispec, exp["bispec"]) <= 1e-5
    assert np.array_equal(fl, exp["flags"])
    d = phase_err(ph, exp["phases"], exp["flags"] > 0)
    assert d.max() <= 1e-3 and np.sqrt((d ** 2).mean()) <= 1e-4, (d.max(), np.sqrt((d ** 2).mean()))
    assert rel_l2(img, exp["image"]) <= 1e-4


@pytest.mark.parametrize("W,H,D", [(99, 75, 14), (37, 64, 8), (60, 45, 16), (30, 17, 10)])
def test_generic_size_accumulate_fft(smip, oracle, W, H, D):
    """Bispectrum::accumulate_from_fft on spectra of odd and mixed sizes
    against FP64; elements the reference never writes stay zero."""
    rng = np.random.default_rng(W + 5 * H + D)
    spec = np.fft.fft2(rng.integers(0, 4096, (5, H, W)).astype(float), axes=(1, 2))
    d = bispec_desc(W, H, D)
    B64 = np.zeros(d["base_size"], np.complex128)
    for f in range(5):
        oracle.accumulate(B64, spec[f], D, fp64=True)
    with smip.Stack(W, H, D, batch_frames=16) as st:
        st.accumulate_from_fft(spec[:3])
        st.accumulate_from_fft(spec[3:])
        got = st.bispectrum()
    assert rel_l2(got, B64 / 5) <= 1e-5
    assert np.all(got[B64 == 0] == 0)


@pytest.mark.parametrize("W,H", [(100, 60), (45, 45), (640, 33)])
def test_generic_size_cross_correlation(smip, oracle, W, H):
    """CrossCorrelation::get_displacement at sizes FFTW plans directly:
    the integer shift equals the oracle's (FP64 correlation, first maximum)."""
    rng = np.random.default_rng(W * H)
    ref = rng.integers(0, 3000, (H, W)).astype(np.float64)
    for dx, dy in ((3, -2), (-7, 5), (0, 0), (W // 2, -(H // 2))):
        frame = oracle.shifted(ref, dx, dy) + rng.integers(0, 40, (H, W))
        assert smip.CrossCorrelation(ref)(frame) == oracle.xcorr(ref, frame)
