"""The allocation-free shift entry point (smip_xcorr_displacement_noalloc).

It serves callers that cannot allocate device memory while they run (fixed
acquisition buffers, host applications that own device memory through their
own pool), so its scratch lives in one fixed array inside the library.  These
tests call it through the C ABI and check its result against the allocating
entry point (smip_xcorr_displacement) on the same inputs, for two calls in a
row on the same array, including a smaller frame after a larger one.  This
file is named to run last so a failure here does not stop earlier tests.
"""
import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu


def _noalloc_shift(smip, torch, ref, frame):
    r = torch.from_numpy(np.ascontiguousarray(ref, np.float64)).cuda()
    f = torch.from_numpy(np.ascontiguousarray(frame, np.float64)).cuda()
    out = torch.full((2,), -12345, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    smip.xcorr_displacement_noalloc(r.data_ptr(), f.data_ptr(), ref.shape[1], ref.shape[0], out.data_ptr(),
                                    stream.cuda_stream)
    stream.synchronize()
    return tuple(int(v) for v in out.cpu().tolist())


def test_no_alloc_matches_allocating_entry_point(smip, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    # two calls in a row: a 256x256 speckle-like frame, then the 128x128 Gaussian
    # of the reference's correl_test with a known shift
    base = rng.integers(0, 4000, (256, 256)).astype(np.float64)
    frame1 = np.roll(base, (17, -23), axis=(0, 1)) + rng.integers(0, 50, (256, 256))
    g = golden("xcorr_gauss")["gaus"]
    frame2 = oracle.shifted(g, 9, -14)
    cases = [(base, frame1), (g, frame2)]
    for ref, frame in cases:
        expected = smip.CrossCorrelation(ref)(frame)
        got = _noalloc_shift(smip, torch, ref, frame)
        assert got == expected, (got, expected)
    assert _noalloc_shift(smip, torch, g, frame2) == (9, -14)


def test_no_alloc_rejects_frames_beyond_its_array(smip):
    torch = pytest.importorskip("torch")
    a = torch.zeros((512, 512), dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(smip.Unsupported, match="256"):
        smip.xcorr_displacement_noalloc(a.data_ptr(), a.data_ptr(), 512, 512, out.data_ptr())
