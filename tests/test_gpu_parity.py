"""GPU parity: libsmip_gpu.so (through its C ABI) against the reference's
fixtures and the CPU oracle on the same seeded frames.

Tolerances (targets: SAA shifts bit-exact, phases within 1e-3 rad of FP64):
  shifts, shift-and-add sum, phase-map flags ............ bit-exact
  power spectrum ........ max |dP| <= 1e-6 max P, rel-L2 <= 1e-6
  bispectrum (normalised) rel-L2 <= 1e-5 against the FP64 oracle
  phases ................ max |dphi| <= 1e-3 rad, RMS <= 1e-4 rad (flagged points)
  image ................. rel-L2 <= 1e-4
"""
import numpy as np
import pytest
from conftest import golden, phase_err, rel_l2

from oracle import bispec_desc

pytestmark = pytest.mark.gpu

PHASE_MAX, PHASE_RMS = 1e-3, 1e-4


def run_gpu(smip, frames, depth, radius, batch=0):
    n, nr, nc = frames.shape
    with smip.Stack(nc, nr, depth, batch_frames=batch) as st:
        st.push_frames(frames)
        out = {"shifts": st.shifts(), "sum": st.sum(), "power": st.power(), "bispec": st.bispectrum()}
        out["image"], out["phases"], out["flags"], out["consistency"] = st.finish(radius)
    return out


def check_against(out, exp, fp64_bispec=None):
    assert np.array_equal(out["shifts"], exp["shifts"])
    assert np.array_equal(out["sum"].view(np.uint64), np.asarray(exp["sum"]).view(np.uint64))
    p_exp = np.real(exp["power"])
    assert np.abs(out["power"] - p_exp).max() <= 1e-6 * p_exp.max()
    assert rel_l2(out["power"], p_exp) <= 1e-6
    assert np.array_equal(out["flags"], exp["flags"])
    m = exp["flags"] > 0
    d = phase_err(out["phases"], exp["phases"], m)
    assert d.max() <= PHASE_MAX, d.max()
    assert np.sqrt((d ** 2).mean()) <= PHASE_RMS
    assert rel_l2(out["image"], exp["image"]) <= 1e-4
    if fp64_bispec is not None:
        assert rel_l2(out["bispec"], fp64_bispec) <= 1e-5


@pytest.mark.parametrize("name", ["stack_binary32_u8", "stack_ext64_u16"])
def test_reference_fixtures(smip, name):
    fx = golden(name)
    out = run_gpu(smip, fx["frames"], int(fx["bdepth"]), float(fx["reco_radius"]))
    check_against(out, fx)
    assert rel_l2(out["bispec"][fx["bispec_sample_idx"]], fx["bispec_sample"]) <= 1e-5
    if "bispec" in fx:
        assert rel_l2(out["bispec"], fx["bispec"]) <= 1e-5


def test_binary128_full_workload(smip, oracle):
    """40 frames of 128x128 u8 binary star, -b 32 -p 64, against the FP64 oracle."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec("binary128")
    frames = S.make_stack(spec)
    exp = oracle.run_stack(frames, spec.bdepth, spec.reco_radius, fp64=True, nthreads=16)
    out = run_gpu(smip, frames, spec.bdepth, spec.reco_radius)
    check_against(out, exp, fp64_bispec=exp["bispec"])
    ref32 = oracle.run_stack(frames, spec.bdepth, spec.reco_radius, fp64=False, nthreads=16)
    assert np.array_equal(out["shifts"], ref32["shifts"])
    assert np.array_equal(out["flags"], ref32["flags"])


def test_extended256_sample(smip, oracle):
    """16 frames of the 256x256 u16 extended-object workload, -b 32 -p 128,
    against the FP64 oracle (the headline shape)."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec("extended256", nframes=16)
    frames = S.make_stack(spec)
    exp = oracle.run_stack(frames, spec.bdepth, spec.reco_radius, fp64=True, nthreads=16)
    out = run_gpu(smip, frames, spec.bdepth, spec.reco_radius, batch=8)
    check_against(out, exp, fp64_bispec=exp["bispec"])


def test_extended512_sample(smip, oracle):
    """4 frames of the 512x512 u16 workload (200 blobs + disk, D/r0 = 25),
    -b 48 -p 200, against the FP64 oracle: the largest frame and the depth-48
    bispectrum tile."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec("extended512", nframes=4)
    frames = S.make_stack(spec)
    exp = oracle.run_stack(frames, spec.bdepth, spec.reco_radius, fp64=True, nthreads=16)
    out = run_gpu(smip, frames, spec.bdepth, spec.reco_radius)
    check_against(out, exp, fp64_bispec=exp["bispec"])


def test_default_depth_pipeline(smip, oracle):
    """smip-cli's default depth -b 20 (not a multiple of 8) through the whole
    pipeline, 128x128 u8 binary star, against the FP64 oracle."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec("binary128", nframes=12)
    frames = S.make_stack(spec)
    exp = oracle.run_stack(frames, 20, 40.0, fp64=True, nthreads=16)
    out = run_gpu(smip, frames, 20, 40.0, batch=8)
    check_against(out, exp, fp64_bispec=exp["bispec"])


@pytest.mark.parametrize("W,H,D", [(16, 16, 8), (32, 64, 16), (64, 32, 24), (64, 64, 32), (128, 64, 40),
                                   (128, 128, 48), (128, 128, 56), (128, 128, 64), (64, 64, 9),
                                   (16, 16, 2), (32, 32, 6), (64, 64, 20), (128, 64, 30), (64, 128, 46)])
def test_accumulate_fft_shapes(smip, oracle, W, H, D):
    """Bispectrum::accumulate_from_fft for every supported depth, rectangular
    frames and an odd depth (behaves as depth-1), against FP64."""
    rng = np.random.default_rng(W * 7 + H * 3 + D)
    spec = np.fft.fft2(rng.integers(0, 4096, (5, H, W)).astype(float), axes=(1, 2))
    d = bispec_desc(W, H, D)
    B64 = np.zeros(d["base_size"], np.complex128)
    for f in range(5):
        oracle.accumulate(B64, spec[f], D, fp64=True)
    with smip.Stack(W, H, D, batch_frames=16) as st:
        st.accumulate_from_fft(spec[:2])
        st.accumulate_from_fft(spec[2:])
        got = st.bispectrum()
        assert st.nframes == 5
    assert rel_l2(got, B64 / 5) <= 1e-5
    # elements the reference never writes stay exactly zero
    assert np.all(got[B64 == 0] == 0)


@pytest.mark.parametrize("W,H,D,n", [(64, 64, 16, 40), (128, 64, 40, 9), (256, 256, 32, 20), (512, 512, 48, 16)])
def test_every_element_accumulated_once(smip, oracle, W, H, D, n):
    """Write-count check of the bispectrum kernel: with every spectrum value
    1 + 0i each in-range triple adds exactly 1 per frame, so the normalised
    bispectrum holds, per packed element, how many times the kernel
    accumulated it -- 1 where the reference's loop (bispectrum.h:393-408)
    writes and 0 elsewhere, exactly.  A tile computed twice, a split part
    merged twice or lost, or a stage read while being refilled shows up as a
    value other than 0 or 1.  At 64x64 with 40 frames (37 tiles, 4 parts each)
    and 512x512 with 16 frames (the last wave's 16 tiles, 2 parts each) tiles
    are split by frames, so the merge of the parts is covered too."""
    ones = np.ones((H, W), np.complex128)
    d = bispec_desc(W, H, D)
    cnt = np.zeros(d["base_size"], np.complex64)  # 0 and 1 are exact in FP32
    oracle.accumulate(cnt, ones, D)
    assert set(np.unique(cnt.real)) <= {0.0, 1.0} and np.all(cnt.imag == 0)
    with smip.Stack(W, H, D) as st:
        st.accumulate_from_fft(np.broadcast_to(ones, (n, H, W)))
        got = st.bispectrum()
    assert np.array_equal(got.real, cnt.real)
    assert np.all(got.imag == 0)


@pytest.mark.parametrize("key", ["n16_d4", "n24_d6", "n32_d8"])
def test_device_get_element_index(smip, key):
    """The device copy of get_element's index path is bit-identical to the
    reference's (aliasing and all) on every pair calc_phase can query."""
    fx = golden("bispec_index")
    n, d = (int(x[1:]) for x in key.split("_"))
    off, cj = smip.bispec_offsets(n, n, d, fx[key + "_idx"])
    assert np.array_equal(off, fx[key + "_off"])
    assert np.array_equal(cj, fx[key + "_conj"])


@pytest.mark.parametrize("W,H,D", [(64, 64, 16), (256, 256, 32), (128, 64, 24), (512, 512, 48)])
def test_device_get_element_vs_oracle(smip, oracle, W, H, D):
    rng = np.random.default_rng(W + D)
    n = 200000 if W < 512 else 50000
    idx = np.stack([rng.integers(-W // 2, W // 2, n), rng.integers(-H // 2, H // 2, n),
                    rng.integers(-D // 2, D // 2 + 1, n), rng.integers(-D // 2, D // 2 + 1, n)], 1).astype(np.int32)
    off, cj = smip.bispec_offsets(W, H, D, idx)
    o2, c2 = oracle.get_element_offsets(W, H, D, idx)
    assert np.array_equal(off, o2) and np.array_equal(cj, c2)


def test_xcorr_gaussian_fixture(smip, oracle):
    """correl_test.cpp restated: every integer shift recovered exactly, as the reference measured."""
    fx = golden("xcorr_gauss")
    g = fx["gaus"]
    cc = smip.CrossCorrelation(g)
    for (dx, dy), m in zip(fx["generated"], fx["measured"]):
        assert cc(oracle.shifted(g, int(dx), int(dy))) == tuple(m)
    assert smip.CrossCorrelation(g).get_displacement(g, oracle.shifted(g, 3, -4)) == (3, -4)


def test_repeat_runs_bit_identical(smip):
    """The same frames give bit-identical results run after run: every output
    of the per-frame pipeline and the phase map.  Catches races between the
    bispectrum kernel's shared-memory ring and its TMA refills."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec("extended256", nframes=24)
    frames = S.make_stack(spec)
    runs = [run_gpu(smip, frames, spec.bdepth, spec.reco_radius, batch=8) for _ in range(3)]
    for r in runs[1:]:
        for key in ("shifts", "sum", "power", "bispec", "phases", "image"):
            assert np.array_equal(np.asarray(r[key]), np.asarray(runs[0][key])), key


def test_merge_equals_single_stack(smip):
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=64, nframes=24, kind="extended", dtype="uint16", d_over_r0=6.0, bdepth=16, seed=9, nblobs=6)
    frames = S.make_stack(spec)
    single = run_gpu(smip, frames, 16, 24, batch=16)
    a = smip.Stack(64, 64, 16, batch_frames=16)
    b = smip.Stack(64, 64, 16, batch_frames=16)
    a.push_frames(frames[:10])
    a.share_reference(b)
    b.push_frames(frames[10:])
    a.merge(b)
    assert a.nframes == 24
    assert np.array_equal(a.shifts(), single["shifts"])
    assert np.array_equal(a.sum(), single["sum"])
    assert rel_l2(a.power(), single["power"]) <= 1e-12
    assert rel_l2(a.bispectrum(), single["bispec"]) <= 1e-6
    img, ph, fl, _ = a.finish(24)
    assert np.array_equal(fl, single["flags"])
    assert phase_err(ph, single["phases"], fl > 0).max() <= PHASE_MAX
    a.close()
    b.close()


def test_batch_size_and_chunking_invariance(smip):
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=64, nframes=37, kind="binary", dtype="uint8", d_over_r0=6.0, bdepth=16, seed=5)
    frames = S.make_stack(spec)
    a = run_gpu(smip, frames, 16, 24, batch=16)
    with smip.Stack(64, 64, 16, batch_frames=32) as st:
        for k in range(0, 37, 5):  # uneven chunks
            st.push_frames(frames[k:k + 5])
        sh, sm, B = st.shifts(), st.sum(), st.bispectrum()
    assert np.array_equal(sh, a["shifts"]) and np.array_equal(sm, a["sum"])
    assert rel_l2(B, a["bispec"]) <= 1e-6


def test_frame_dtypes_agree(smip):
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=32, nframes=10, kind="binary", dtype="uint8", d_over_r0=4.0, bdepth=8, seed=21)
    f8 = S.make_stack(spec)
    outs = [run_gpu(smip, f8.astype(t), 8, 12) for t in (np.uint8, np.uint16, np.float32, np.float64)]
    for o in outs[1:]:
        assert np.array_equal(o["shifts"], outs[0]["shifts"])
        assert np.array_equal(o["sum"], outs[0]["sum"])
        assert rel_l2(o["bispec"], outs[0]["bispec"]) <= 1e-6
        assert np.array_equal(o["flags"], outs[0]["flags"])


def test_reused_stack_across_frame_types(smip):
    """One stack reset between jobs of different frame types -- u8, then u16
    and f64 (larger elements: its staging buffers are replaced), then u8
    again (smaller: the buffers are reused) -- gives, job by job, exactly
    the results of a fresh stack; the reference frame and shift list are
    allocated with the stack, so no job reallocates them."""
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=64, nframes=70, kind="extended", dtype="uint16", d_over_r0=6.0, bdepth=16, seed=29)
    fr = S.make_stack(spec)
    jobs = [(fr[:40] >> 4).astype(np.uint8), fr[10:70], fr[5:50].astype(np.float64), (fr[30:70] >> 4).astype(np.uint8)]

    def results(st, frames):
        st.push_frames(frames)
        img, ph, fl, cs = st.finish(20.0)
        return st.shifts(), st.sum(), st.bispectrum(), img, fl

    with smip.Stack(64, 64, 16, batch_frames=32) as st:
        for frames in jobs:
            got = results(st, frames)
            with smip.Stack(64, 64, 16, batch_frames=32) as fresh:
                exp = results(fresh, frames)
            for g, e in zip(got, exp):
                assert np.array_equal(g, e)
            st.reset()


def test_prepared_reconstruction_matches(smip):
    """prepare_reco allocates and builds the reconstruction's tables ahead of
    finish: the same radius gives identical results, a stack prepared for
    another radius rebuilds them, and a negative radius is refused."""
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=64, nframes=24, kind="extended", dtype="uint16", d_over_r0=6.0, bdepth=16, seed=31)
    fr = S.make_stack(spec)
    outs = []
    for prep in (None, 24.0, 40.0):
        with smip.Stack(64, 64, 16) as st:
            if prep is not None:
                st.prepare_reco(prep)
            st.push_frames(fr)
            outs.append(st.finish(24.0))
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a, b)
    with smip.Stack(64, 64, 16) as st, pytest.raises(smip.InvalidArgument):
        st.prepare_reco(-1.0)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.float32, np.float64])
def test_host_device_and_page_locked_sources_agree(smip, dtype):
    """The same frames pushed from pageable host memory (copied), from
    page-locked host memory (the first full batch read by the row pass
    through the mapped pointer, the rest copied) and from device memory give
    bit-identical results."""
    import torch
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=64, nframes=40, kind="extended", dtype="uint16", d_over_r0=6.0, bdepth=16, seed=23)
    fr = S.make_stack(spec)
    fr = (fr >> 4).astype(dtype) if dtype == np.uint8 else fr.astype(dtype)
    t = torch.from_numpy(fr.view(np.int16) if dtype == np.uint16 else fr)
    pinned = t.pin_memory()
    pinned_np = pinned.numpy().view(dtype)
    dev = t.cuda()
    dev = dev.view(torch.uint16) if dtype == np.uint16 else dev
    outs = []
    for src in (fr, pinned_np, dev):
        with smip.Stack(64, 64, 16, batch_frames=16) as st:
            st.push_frames(src)
            o = {"shifts": st.shifts(), "sum": st.sum(), "power": st.power(), "bispec": st.bispectrum()}
            o["image"], o["phases"], o["flags"], _ = st.finish(20.0)
        outs.append(o)
    for o in outs[1:]:
        for k in o:
            assert np.array_equal(o[k], outs[0][k]), k


@pytest.mark.parametrize("name,nframes", [("binary128", 40), ("extended256", 16)])
def test_ring_mode_estimator(smip, oracle, name, nframes):
    """The opt-in ring-parallel estimator on the same stack as the spiral
    walk: the same points get phases, the reconstructed image's magnitude
    stays within 1 % (rel-L2) of the FP64 oracle's (measured: 0.5 % at 128²,
    0.2 % at 256²), repeat runs are bit-identical, and switching back gives
    the spiral's results exactly."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec(name, nframes=nframes)
    frames = S.make_stack(spec)
    n, R = frames.shape[1], float(spec.reco_radius)
    exp = oracle.run_stack(frames, spec.bdepth, R, fp64=True, nthreads=16)
    with smip.Stack(n, n, spec.bdepth) as st:
        st.push_frames(frames)
        sp = st.finish(R)
        st.set_reco_mode("rings")
        r1 = st.finish(R)
        r2 = st.finish(R)
        st.set_reco_mode("spiral")
        sp2 = st.finish(R)
    for a, b in zip(r1, r2):
        assert np.array_equal(a, b)
    for a, b in zip(sp, sp2):
        assert np.array_equal(a, b)
    assert np.array_equal(r1[2], exp["flags"])
    assert rel_l2(np.abs(r1[0]), np.abs(exp["image"])) <= 1e-2
    with pytest.raises(smip.InvalidArgument):
        with smip.Stack(n, n, spec.bdepth) as st:
            st.set_reco_mode(7)


def test_single_frame_and_errors(smip, oracle):
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=32, nframes=1, kind="binary", dtype="uint8", d_over_r0=4.0, bdepth=8, seed=2)
    f = S.make_stack(spec)
    out = run_gpu(smip, f, 8, 12)
    exp = oracle.run_stack(f, 8, 12)
    check_against(out, exp)
    with smip.Stack(32, 32, 8) as st:
        with pytest.raises(smip.RuntimeFailure):
            st.bispectrum()  # division by zero: no frames
        st.push_frames(f)
        with pytest.raises(smip.InvalidArgument):
            st.push_frames(f.astype(np.uint16))
        with pytest.raises(smip.InvalidArgument):
            st.accumulate_from_fft(np.zeros((1, 32, 32), np.complex128))
        with pytest.raises(smip.OutOfRange):
            st.shifts(0, 5)
        with pytest.raises(smip.DomainError):
            st.finish(0.0)
    with smip.Stack(32, 32, 8) as st:
        st.accumulate_from_fft(np.fft.fft2(f[0].astype(float)))
        with pytest.raises(smip.BadFunctionCall):
            st.finish(12)
        ph, fl, _ = st.reconstruct_phases(12)  # phases need only the bispectrum
        assert fl.sum() > 5


def test_standalone_reconstruct_phases(smip, oracle):
    fx = golden("stack_binary32_u8")
    ph, fl, cs = smip.reconstruct_phases(fx["bispec"], 32, 32, 8, float(fx["reco_radius"]))
    assert np.array_equal(fl, fx["flags"])
    assert phase_err(ph, fx["phases"], fl > 0).max() <= PHASE_MAX
    assert np.abs(cs - fx["consistency"]).max() <= 1e-5


def test_shifted_matches_oracle(smip, oracle):
    """Array2<double>::shifted for shifts inside the array, edges included,
    against the oracle's restatement of array2.h:603-622; a distance as large
    as the array (where the reference reads outside it) is OutOfRange."""
    rng = np.random.default_rng(11)
    a = rng.normal(size=(32, 64))
    for dx, dy in [(0, 0), (3, -5), (-17, 9), (63, 31), (-63, -31), (1, 0), (0, -1)]:
        assert np.array_equal(smip.shifted(a, dx, dy), oracle.shifted(a, dx, dy)), (dx, dy)
    with pytest.raises(smip.OutOfRange):
        smip.shifted(a, 64, 0)
    with pytest.raises(smip.OutOfRange):
        smip.shifted(a, 0, -32)


def test_hann_matches_reference_formula(smip, oracle):
    assert np.abs(smip.hann(64, 32, 48.0) - oracle.hann(64, 32, 48.0)).max() <= 1e-15


def test_save_bispectrum_format(smip, tmp_path):
    fx = golden("stack_binary32_u8")
    with smip.Stack(32, 32, 8) as st:
        st.push_frames(fx["frames"])
        fn = str(tmp_path / "bispectrum.dat")
        st.save_bispectrum(fn)
        B = st.bispectrum()
    raw = open(fn, "rb").read()
    hdr = np.frombuffer(raw[:40], np.uint64)
    assert list(hdr) == [B.size, 32, 32, 8, 8]
    assert np.array_equal(np.frombuffer(raw[40:], np.complex64), B)


def test_load_bispectrum_resume(smip, tmp_path):
    """bispectrum.dat written by one stack and read back into another: the
    phase map is identical, and accumulation resumes where it stopped."""
    rng = np.random.default_rng(7)
    W = H = 64
    D = 16
    spec = np.fft.fft2(rng.integers(0, 4096, (6, H, W)).astype(float), axes=(1, 2))
    fn = str(tmp_path / "bispectrum.dat")
    with smip.Stack(W, H, D) as a:
        a.accumulate_from_fft(spec[:4])
        a.save_bispectrum(fn)
        ph_a, fl_a, _ = a.reconstruct_phases(20)
        b4 = a.bispectrum()
        a.accumulate_from_fft(spec[4:])
        b6 = a.bispectrum()
    with smip.Stack(W, H, D) as b:
        b.load_bispectrum(fn)
        assert b.nframes == 1
        assert np.array_equal(b.bispectrum(), b4)
        ph_b, fl_b, _ = b.reconstruct_phases(20)
        assert np.array_equal(fl_b, fl_a) and np.array_equal(ph_b, ph_a)
    with smip.Stack(W, H, D) as c:
        c.load_bispectrum(fn, nframes=4)
        c.accumulate_from_fft(spec[4:])
        assert c.nframes == 6
        assert rel_l2(c.bispectrum(), b6) <= 1e-6
        with pytest.raises(smip.InvalidArgument):
            c.push_frames(np.zeros((1, H, W), np.uint16))
    with smip.Stack(W, H, D) as m:  # the same from memory
        m.set_bispectrum(b4)
        assert np.array_equal(m.bispectrum(), b4)
        ph_m, fl_m, _ = m.reconstruct_phases(20)
        assert np.array_equal(fl_m, fl_a) and np.array_equal(ph_m, ph_a)
    with smip.Stack(W, H, 24) as d, pytest.raises(smip.InvalidArgument):
        d.load_bispectrum(fn)
    with smip.Stack(W, H, D) as e, pytest.raises(smip.RuntimeFailure):
        e.load_bispectrum(str(tmp_path / "missing.dat"))


def test_stack_state_checkpoint_resume(smip, tmp_path):
    """A job stopped after 30 frames (save_state) and resumed in another stack
    (load_state) gives bit-identical shifts, sums, power, bispectrum and phases
    to the uninterrupted job (the batches line up: 10 frames each)."""
    rng = np.random.default_rng(9)
    base = rng.integers(0, 4096, (64, 64))
    moves = rng.integers(-5, 6, (50, 2))
    frames = (np.stack([np.roll(base, (int(dy), int(dx)), axis=(0, 1)) for dx, dy in moves])
              + rng.integers(0, 50, (50, 64, 64))).astype(np.uint16)

    def results(st):
        ph, fl, _ = st.reconstruct_phases(20)
        return st.shifts(), st.sum(), st.power(), st.bispectrum(), ph, fl

    with smip.Stack(64, 64, 16, batch_frames=10) as a:
        a.push_frames(frames)
        full = results(a)
    fn = str(tmp_path / "job.state")
    with smip.Stack(64, 64, 16, batch_frames=10) as b:
        b.push_frames(frames[:30])
        b.save_state(fn)
    with smip.Stack(64, 64, 16, batch_frames=10) as c:
        c.load_state(fn)
        assert c.nframes == 30
        c.push_frames(frames[30:])
        resumed = results(c)
    for x, y in zip(full, resumed):
        assert np.array_equal(x, y)
    with smip.Stack(32, 32, 16) as d, pytest.raises(smip.InvalidArgument):
        d.load_state(fn)


def test_weak_bins_keep_fp32_accuracy(smip):
    """The forward FFT is float-float: every power-spectrum bin down to 1e-8 of
    the strongest keeps 1e-6 relative accuracy against an FP64 FFT of the same
    256x256 u16 speckle frame (a plain FP32 FFT is off by ~1e-2 there)."""
    from smip_gb300 import synthetic as S

    fr = S.make_stack(S.config_spec("extended256", nframes=1), 0, 1)
    with smip.Stack(256, 256, 32) as st:
        st.push_frames(fr)
        P = st.power()
    F2 = np.abs(np.fft.fft2(fr[0].astype(np.float64))) ** 2 / fr[0].size
    m = F2 >= 1e-8 * F2.max()
    rel = np.abs(P[m] - F2[m]) / F2[m]
    assert rel.max() <= 1e-6, rel.max()


def test_full_size_properties(smip):
    """256x256 u16, depth 32, 64 frames: size-independent checks against
    float64 numpy on the same frames (no oracle at this size)."""
    from smip_gb300 import synthetic as S

    spec = S.config_spec("extended256", nframes=64)
    base = S.make_stack(spec, 0, 1)[0]
    rng = np.random.default_rng(1)
    true = rng.integers(-40, 40, (64, 2))
    true[0] = 0
    frames = np.stack([np.roll(base, (dy, dx), axis=(0, 1)) for dx, dy in true]) \
        + rng.integers(0, 3, (64, 256, 256)).astype(np.uint16)
    with smip.Stack(256, 256, 32) as st:
        st.push_frames(frames)
        sh, sm, P, B = st.shifts(), st.sum(), st.power(), st.bispectrum()
    # circularly shifted copies: the correlation peak is at the true shift
    assert np.array_equal(sh, true)
    # shift-and-add sum reproduced exactly in integers with those shifts
    acc = frames[0].astype(np.int64)
    for f in range(1, 64):
        dx, dy = sh[f]
        s = np.zeros((256, 256), np.int64)
        ys, xs = slice(max(0, -dy), min(256, 256 - dy)), slice(max(0, -dx), min(256, 256 - dx))
        yd, xd = slice(max(0, -dy) + dy, min(256, 256 - dy) + dy), slice(max(0, -dx) + dx, min(256, 256 - dx) + dx)
        s[ys, xs] = frames[f][yd, xd]
        acc += s
    assert np.array_equal(sm, acc / 64.0)
    # Parseval: sum_k P(k) = mean_f sum_x f^2
    e = (frames.astype(np.float64) ** 2).sum(axis=(1, 2)).mean()
    assert abs(P.sum() - e) <= 1e-6 * e
    # B(0,0,0,0) = mean F(0)^3 and B(u, v=0) = mean |F(u)|^2 F(0)
    F = np.fft.fft2(frames.astype(np.float64), axes=(1, 2))
    b000 = (F[:, 0, 0] ** 3).mean()
    assert abs(B[0] - b000) <= 1e-5 * abs(b000)
    # element (u=(-3,5), v=(0,0)): a0=3, a1=5, a2=0, a3=0
    off = ((3 * 257 + 5) * 17 + 0) * 33 + 0
    u = F[:, 5, -3]
    exp = (u * F[:, 0, 0] * np.conj(u)).mean()
    assert abs(B[off] - exp) <= 1e-5 * abs(exp)
