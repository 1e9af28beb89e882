"""GPU parity at the lengths the benchmark times.

The benchmark accumulates 2000 frames of 256x256 in batches of 1024 + 976
frames; inside a batch each triple sum stays in FP32 registers (Kahan
compensation applies across batches).  These tests run exactly that, and one
whole 288-frame batch at 512x512 (depth 48, radius 200, the largest
configuration), against the FP64 oracle on the same seeded frames:

  shifts, shift-and-add sum, phase-map flags ............ bit-exact
  power spectrum ........ max |dP| <= 1e-6 max P
  bispectrum (normalised) rel-L2 <= 1e-5 against FP64
  phases ................ max |dphi| <= 1e-3 rad, RMS <= 1e-4 rad (flagged points)
  image ................. rel-L2 <= 1e-4

and they separate the phase chain's own precision from the accumulation's:
the oracle's FP64 phase recovery (phasereco.h:33-123) run on the bispectrum
the GPU accumulated must agree with the GPU's phase recovery on it within
1e-4 rad (ten times inside the 1e-3 rad target), so any remaining phase
difference comes from the FP32 bispectrum, which the reference also
accumulates in complex<float> (bispectrum.h:399-403).

The measured errors are printed (run with -s to see them).
"""
import json
import os

import numpy as np
import pytest
from conftest import phase_err, rel_l2

pytestmark = pytest.mark.gpu

PHASE_MAX, PHASE_RMS, CHAIN_MAX = 1e-3, 1e-4, 1e-4
THREADS = os.cpu_count() or 1


def _errors(out, exp, fp64_bispec):
    m = exp["flags"] > 0
    d = phase_err(out["phases"], exp["phases"], m)
    p_exp = np.real(exp["power"])
    return {"shifts_bit_exact": bool(np.array_equal(out["shifts"], exp["shifts"])),
            "sum_bit_exact": bool(np.array_equal(out["sum"].view(np.uint64), np.asarray(exp["sum"]).view(np.uint64))),
            "flags_identical": bool(np.array_equal(out["flags"], exp["flags"])),
            "phase_max_rad": float(d.max()), "phase_rms_rad": float(np.sqrt((d ** 2).mean())),
            "power_max_rel": float(np.abs(out["power"] - p_exp).max() / p_exp.max()),
            "bispectrum_rel_l2": rel_l2(out["bispec"], fp64_bispec),
            "image_rel_l2": rel_l2(out["image"], exp["image"])}


def _run_full(smip, oracle, name, nframes, batch):
    from smip_gb300 import synthetic as S

    spec = S.config_spec(name, nframes=nframes)
    frames = S.make_stack(spec, procs=min(16, THREADS))
    exp = oracle.run_stack(frames, spec.bdepth, spec.reco_radius, fp64=True, nthreads=THREADS)
    n = spec.n
    R = float(spec.reco_radius)
    with smip.Stack(n, n, spec.bdepth, batch_frames=batch) as st:
        st.set_timing(True)
        st.push_frames(frames)
        st.flush()
        _, launches, kframes = st.kernel_time()
        out = {"shifts": st.shifts(), "sum": st.sum(), "power": st.power(), "bispec": st.bispectrum()}
        out["image"], out["phases"], out["flags"], out["consistency"] = st.finish(R)
    # the oracle's FP64 phase recovery on the GPU's own (normalised FP32) bispectrum
    ph_o, fl_o, _ = oracle.reconstruct_phases(out["bispec"], n, n, spec.bdepth, R)
    chain = phase_err(out["phases"], ph_o, fl_o > 0)
    err = _errors(out, exp, exp["bispec"])
    err.update({"workload": f"{nframes} x {n}x{n}, d{spec.bdepth}, R{spec.reco_radius:g}",
                "batches": launches, "frames_accumulated": kframes,
                "chain_flags_identical": bool(np.array_equal(out["flags"], fl_o)),
                "chain_phase_max_rad": float(chain.max()),
                "chain_phase_rms_rad": float(np.sqrt((chain ** 2).mean()))})
    print(json.dumps(err))
    return err


def _check(err):
    assert err["shifts_bit_exact"] and err["sum_bit_exact"] and err["flags_identical"], err
    assert err["power_max_rel"] <= 1e-6, err
    assert err["bispectrum_rel_l2"] <= 1e-5, err
    assert err["phase_max_rad"] <= PHASE_MAX and err["phase_rms_rad"] <= PHASE_RMS, err
    assert err["image_rel_l2"] <= 1e-4, err
    assert err["chain_flags_identical"], err
    assert err["chain_phase_max_rad"] <= CHAIN_MAX, err


def test_extended256_whole_stack(smip, oracle):
    """The whole 2000-frame 256x256 u16 stack (-b 32 -p 128) in the benchmark's
    batches: 1024 frames summed in registers, then 976."""
    err = _run_full(smip, oracle, "extended256", 2000, 1024)
    assert err["batches"] == 2 and err["frames_accumulated"] == 2000
    _check(err)


def test_extended512_full_batch(smip, oracle):
    """One whole 288-frame batch (the library's batch at 512x512) of the
    512x512 u16 workload (-b 48 -p 200) plus 12 frames in a second batch."""
    err = _run_full(smip, oracle, "extended512", 300, 0)
    assert err["batches"] == 2 and err["frames_accumulated"] == 300
    _check(err)
