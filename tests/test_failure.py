"""Failure detection without a GPU fault: every device-side wait of the
kernels is bounded, and an expired wait is recorded on the device and reported
by the next call (SMIP_E_TIMEOUT -> DeviceTimeout).  smip_diag_bounded_wait
runs that path on purpose: a kernel waits on an mbarrier nothing arrives on
and on a flag nothing sets, both give up after the limit and return."""
import time

import numpy as np
import pytest


def test_diag_rejects_bad_limits(smip):
    for t in (0.0, -1.0, 11.0):
        with pytest.raises(smip.InvalidArgument):
            smip.diag_bounded_wait(0, t)


@pytest.mark.gpu
def test_expired_wait_is_reported_and_device_stays_usable(smip):
    t0 = time.perf_counter()
    with pytest.raises(smip.DeviceTimeout):
        smip.diag_bounded_wait(0, 0.05)
    assert time.perf_counter() - t0 < 5.0
    # the context is intact: a stack runs and a second probe reports again
    rng = np.random.default_rng(2)
    frames = rng.integers(0, 4096, (6, 32, 32)).astype(np.uint16)
    frames[3:] = np.roll(frames[:3], (2, -1), axis=(1, 2))
    with smip.Stack(32, 32, 8) as st:
        st.push_frames(frames)
        st.sync()
        assert st.nframes == 6
    with pytest.raises(smip.DeviceTimeout):
        smip.diag_bounded_wait(0, 0.02)
