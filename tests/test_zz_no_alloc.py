"""The allocation-free shift entry point (smip_xcorr_displacement_noalloc).

It serves callers that cannot allocate device memory while they run (fixed
acquisition buffers, host applications that own device memory through their
own pool), so its scratch lives in one fixed array inside the library.  These
tests call it through the C ABI and check its result against the allocating
entry point (smip_xcorr_displacement) on the same inputs, for calls in a row
on the same array (square and rectangular frames, a smaller frame after a
larger one), and that calls after the first leave the device's free memory
and torch's allocations unchanged.  This file is named to run last so a
failure here does not stop earlier tests.
"""
import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu


def _cases(oracle):
    rng = np.random.default_rng(77)
    # a 256x256 speckle-like frame, the 128x128 Gaussian of the reference's
    # correl_test with a known shift, and two rectangular frames
    base = rng.integers(0, 4000, (256, 256)).astype(np.float64)
    frame1 = np.roll(base, (17, -23), axis=(0, 1)) + rng.integers(0, 50, (256, 256))
    g = golden("xcorr_gauss")["gaus"]
    frame2 = oracle.shifted(g, 9, -14)
    rect = rng.integers(0, 4000, (64, 128)).astype(np.float64)   # 64 rows x 128 columns
    frame3 = oracle.shifted(rect, -5, 11) + rng.integers(0, 30, (64, 128))
    tall = rng.integers(0, 4000, (256, 32)).astype(np.float64)   # 256 rows x 32 columns
    frame4 = oracle.shifted(tall, 3, -40) + rng.integers(0, 30, (256, 32))
    return [(base, frame1), (g, frame2), (rect, frame3), (tall, frame4)]


def test_no_alloc_matches_allocating_entry_point(smip, oracle):
    torch = pytest.importorskip("torch")
    cases = _cases(oracle)
    expected = [smip.CrossCorrelation(ref)(frame) for ref, frame in cases]
    dev = [(torch.from_numpy(np.ascontiguousarray(r)).cuda(), torch.from_numpy(np.ascontiguousarray(f)).cuda())
           for r, f in cases]
    outs = [torch.full((2,), -12345, dtype=torch.int32, device="cuda") for _ in range(2 * len(cases))]
    stream = torch.cuda.current_stream()

    def call(k, out):
        r, f = dev[k]
        smip.xcorr_displacement_noalloc(r.data_ptr(), f.data_ptr(), r.shape[1], r.shape[0], out.data_ptr(),
                                        stream.cuda_stream)
        stream.synchronize()

    # the first call on the device sets the array up (it may allocate then)
    warm = torch.zeros(2, dtype=torch.int32, device="cuda")
    call(1, warm)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    # every case twice in a row, largest first, so each later call reuses what
    # a different earlier call left in the shared array
    for rep in range(2):
        for k in range(len(cases)):
            call(k, outs[rep * len(cases) + k])
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert torch.cuda.memory_allocated() == alloc0
    for rep in range(2):
        for k in range(len(cases)):
            got = tuple(int(v) for v in outs[rep * len(cases) + k].cpu().tolist())
            assert got == expected[k], (rep, k, got, expected[k])
    assert expected[1] == (9, -14)


def test_no_alloc_rejects_frames_beyond_its_array(smip):
    torch = pytest.importorskip("torch")
    a = torch.zeros((512, 512), dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(smip.Unsupported, match="256"):
        smip.xcorr_displacement_noalloc(a.data_ptr(), a.data_ptr(), 512, 512, out.data_ptr())
    b = torch.zeros((256, 384), dtype=torch.float64, device="cuda")
    with pytest.raises(smip.Unsupported, match="256"):
        smip.xcorr_displacement_noalloc(b.data_ptr(), b.data_ptr(), 384, 256, out.data_ptr())
