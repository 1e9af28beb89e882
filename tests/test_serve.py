"""Batched/served execution (smip_gb300/serve.py): admission by bispectrum
bytes, continuous batching, and -- on the GPU -- that every job's results are
the same alone and in a mix."""
import numpy as np
import pytest

from smip_gb300 import serve


class FakeStack:
    """Host stand-in for smip_gb300.Stack: records pushes, returns a result
    that depends only on the job's own frames."""

    live = 0

    def __init__(self, nc, nr, d):
        self.shape = (nc, nr, d)
        self.frames = []
        FakeStack.live += 1

    def push_frames(self, f):
        self.frames.append(np.array(f))

    def finish(self, R):
        a = np.concatenate(self.frames).astype(np.float64)
        s = a.sum(axis=0) + R
        return s.astype(np.complex128), s.astype(np.complex128), (s > 0).astype(np.uint8), s

    def shifts(self):
        return np.zeros((sum(len(f) for f in self.frames), 2), np.int32)

    def reset(self):
        self.frames = []

    def set_reco_mode(self, mode):
        self.mode = mode


def _jobs(n, rate=None, seed=1):
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for i in range(n):
        sz = int(rng.choice([16, 32]))
        fr = rng.integers(0, 255, (int(rng.integers(3, 70)), sz, sz)).astype(np.uint8)
        if rate:
            t += float(rng.exponential(1.0 / rate))
        out.append(serve.Job(i, fr, 8, 6.0, arrival=t if rate else 0.0, chunk=16))
    return out


def test_bispectrum_bytes_matches_layout():
    from oracle import bispec_desc

    for n, d in ((64, 16), (128, 24), (256, 32), (64, 9)):
        assert serve.bispectrum_bytes(n, n, d) == 3 * 8 * bispec_desc(n, n, d)["base_size"]


def test_engine_admission_and_results():
    jobs = _jobs(20)
    budget = 3 * serve.bispectrum_bytes(32, 32, 8)  # at most three jobs' bispectra
    eng = serve.Engine(budget_bytes=budget, max_active=8, workers=2, stack_factory=FakeStack)
    res, span = eng.run(jobs, realtime=False)
    assert sorted(r.id for r in res) == list(range(20))
    assert eng.peak_bytes <= budget and eng.peak_active <= 8
    plain, _ = serve.run_plain(jobs, realtime=False, stack_factory=FakeStack)
    by_id = {r.id: r for r in plain}
    for r in res:
        assert np.array_equal(r.image, by_id[r.id].image) and r.nframes == len(jobs[r.id].frames)
    s = serve.summarize(res, span)
    assert s["jobs"] == 20 and s["frames"] == sum(len(j.frames) for j in jobs)


def test_engine_graph_mode_launches_each_finished_job_once():
    """With graph=True the stacks of the jobs whose frames are all in after a
    round are handed to one batch launch before their reconstructions."""
    jobs = _jobs(12)
    calls = []

    def launch(stacks, reserve_sms=0):
        assert all(len(st.frames) for st in stacks)  # every one holds its job's frames
        calls.append(([id(st) for st in stacks], reserve_sms))

    eng = serve.Engine(max_active=5, workers=2, stack_factory=FakeStack, graph=True, batch_launch=launch,
                       graph_group=2, graph_reserve=7)
    res, _ = eng.run(jobs, realtime=False)
    assert sorted(r.id for r in res) == list(range(12))
    assert sum(len(c) for c, _ in calls) == 12 and all(len(set(c)) == len(c) <= 2 for c, _ in calls)
    # the first launch has no reconstruction beside it; a group after the first in a round has
    assert calls[0][1] == 0 and calls[1][1] == 7 and {r for _, r in calls} <= {0, 7}


def test_engine_realtime_respects_arrivals():
    jobs = _jobs(8, rate=200.0)
    eng = serve.Engine(max_active=4, workers=2, stack_factory=FakeStack)
    res, _ = eng.run(jobs, realtime=True)
    for r in res:
        assert r.admitted >= r.arrival - 1e-9 and r.done >= r.admitted


def test_prewarm_prepares_reconstructions():
    """prewarm(reco_radius=...) prepares every pooled stack of a shape for the
    radius its jobs use (a function of the shape, or one number); stacks
    without prepare_reco are left as they are."""

    class PreparingStack(FakeStack):
        def prepare_reco(self, R):
            self.prepared = R

    eng = serve.Engine(max_active=2, workers=1, stack_factory=PreparingStack)
    eng.prewarm({(32, 32, 8), (16, 16, 4)}, count=3, reco_radius=lambda shape: 2.0 * shape[2])
    assert {st.prepared for st in eng.pool[(32, 32, 8)]} == {16.0}
    assert {st.prepared for st in eng.pool[(16, 16, 4)]} == {8.0} and len(eng.pool[(16, 16, 4)]) == 3
    eng.prewarm({(16, 16, 4)}, count=4, reco_radius=5.0)
    assert {st.prepared for st in eng.pool[(16, 16, 4)]} == {5.0} and len(eng.pool[(16, 16, 4)]) == 4
    plain = serve.Engine(max_active=2, workers=1, stack_factory=FakeStack)
    plain.prewarm({(16, 16, 4)}, count=2, reco_radius=5.0)  # FakeStack has no prepare_reco
    assert len(plain.pool[(16, 16, 4)]) == 2


def test_engine_pool_reuses_stacks():
    FakeStack.live = 0
    jobs = _jobs(12)
    eng = serve.Engine(max_active=2, workers=1, stack_factory=FakeStack)
    eng.prewarm({j.shape for j in jobs}, count=2)
    made = FakeStack.live
    eng.run(jobs, realtime=False)
    assert FakeStack.live == made  # no stack created while serving


@pytest.mark.gpu
def test_results_same_alone_and_in_mix(smip):
    """Jobs of mixed sizes (64^2, 128^2 and 256^2, binary u8 and extended u16,
    uneven counts) served concurrently give exactly the results each gives
    alone."""
    jobs = serve.make_jobs(8, sizes=(64, 128, 256), counts=(30, 300), bank_frames=64, seed=11)
    assert {j.shape[0] for j in jobs} == {64, 128, 256}
    alone, _ = serve.run_plain(jobs, realtime=False)
    by_id = {r.id: r for r in alone}
    for graph in (False, True):  # last batches flushed per job, or one persistent launch per round
        eng = serve.Engine(max_active=8, workers=3, graph=graph)
        eng.prewarm({j.shape for j in jobs}, count=3)
        mixed, _ = eng.run(jobs, realtime=False)
        assert eng.peak_active >= 2
        for r in mixed:
            a = by_id[r.id]
            assert np.array_equal(r.shifts, a.shifts)
            assert np.array_equal(r.flags, a.flags)
            assert np.array_equal(r.phases, a.phases)
            assert np.array_equal(r.image, a.image)


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    """best_config tunes the batch size, then the kernel's staging variant and
    split, once per (device, shape, depth, dtype) and then reads the cache;
    the measurement itself is replaced by a stand-in here."""
    from smip_gb300 import autotune

    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "at.json"))
    monkeypatch.setattr(autotune, "_device_name", lambda d: "dev")
    calls = []

    def fake_measure(nc, nr, d, bf, frames, device=0, repeats=2, kernel=(0, 0)):
        calls.append((bf, kernel))
        return 1000.0 - abs(bf - 256) + (5.0 if kernel == (1, 32) else 0.0)  # best at 256, variant 1, parts >= 32

    monkeypatch.setattr(autotune, "measure", fake_measure)
    assert autotune.best_config(64, 64, 16, np.uint8) == {"batch_frames": 256, "variant": 1, "min_part": 32}
    assert autotune.best_batch(64, 64, 16, np.uint8) == 256
    n = len(calls)
    assert n == len(autotune.CANDIDATES) + len(autotune.KERNEL_CANDIDATES)
    assert all(bf == 256 for bf, _ in calls[len(autotune.CANDIDATES):])  # kernel tunables at the best batch
    assert autotune.best_batch(64, 64, 16, np.uint8) == 256 and len(calls) == n  # cached
    assert autotune.best_batch(64, 64, 17, np.uint8) == 256 and len(calls) == n  # depth 17 acts as 16
    autotune.best_batch(64, 64, 16, np.uint16)
    assert len(calls) == 2 * n


@pytest.mark.gpu
def test_autotune_on_device(smip, tmp_path, monkeypatch):
    """A real (small) tuning run picks one of the candidates and the stack it
    configures gives the same bispectrum as the default batch size; the two
    staging variants give the same bits."""
    from smip_gb300 import autotune

    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "at.json"))
    monkeypatch.setattr(autotune, "CANDIDATES", (16, 32, 64))
    cfg = autotune.best_config(32, 32, 8, np.uint8)
    assert cfg["batch_frames"] in (16, 32, 64) and (cfg["variant"], cfg["min_part"]) in autotune.KERNEL_CANDIDATES
    rng = np.random.default_rng(3)
    frames = rng.integers(0, 255, (40, 32, 32)).astype(np.uint8)
    with smip.Stack(32, 32, 8, batch_frames="auto", dtype=np.uint8) as a, smip.Stack(32, 32, 8) as b:
        a.push_frames(frames)
        b.push_frames(frames)
        assert np.array_equal(a.shifts(), b.shifts())
        from conftest import rel_l2

        assert rel_l2(a.bispectrum(), b.bispectrum()) <= 1e-6
    rng = np.random.default_rng(4)
    frames = rng.integers(0, 4095, (70, 128, 96)).astype(np.uint16)
    out = []
    for variant, min_part in ((0, 0), (1, 0), (0, 1 << 30)):
        with smip.Stack(96, 128, 24, batch_frames=64) as st:
            st.set_kernel_config(variant, min_part)
            st.push_frames(frames)
            out.append(st.bispectrum())
    assert np.array_equal(out[0], out[1])  # staging does not change the order of the sums
    assert rel_l2(out[2], out[0]) <= 1e-6  # an unsplit last wave sums in another order


@pytest.mark.gpu
def test_batch_launch_matches_flush(smip):
    """One persistent bispectrum launch over the pending batches of several
    stacks (uneven shapes, depths and counts, an odd frame size, a depth that
    is not a multiple of 8; some batches already launched on their own) gives
    bit-identical results to flushing each stack, over repeated calls that
    reuse the captured graphs."""
    rng = np.random.default_rng(5)
    cfg = [(64, 64, 16, 50), (128, 128, 24, 130), (64, 64, 16, 70), (256, 256, 32, 40), (64, 64, 16, 64),
           (99, 75, 20, 45), (48, 48, 8, 30)]
    frames = [rng.integers(0, 4096, (nf, h, w)).astype(np.uint16) for w, h, d, nf in cfg]

    def results(st):
        return st.shifts(), st.sum(), st.power(), st.bispectrum()

    def run(graph):
        stacks = [smip.Stack(w, h, d, batch_frames=64) for w, h, d, _ in cfg]
        out = []
        for rnd in range(3):
            for st, fr in zip(stacks, frames):
                st.reset()
                st.push_frames(fr[rnd:])  # 64 frames run as a batch during the push
            if graph:  # the second round leaves 40 SMs out of the persistent grid
                smip.batch_launch(stacks, reserve_sms=40 if rnd == 1 else 0)
            out.append([results(st) for st in stacks])
        for st in stacks:
            st.close()
        return out

    eager, graphed = run(False), run(True)
    for re, rg in zip(eager, graphed):
        for a, b in zip(re, rg):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)
    with smip.Stack(64, 64, 16) as st:
        st.push_frames(frames[0][:3])
        with pytest.raises(smip.InvalidArgument):
            smip.batch_launch([st, st])
        with pytest.raises(smip.InvalidArgument, match="reserve_sms"):
            smip.batch_launch([st], reserve_sms=100000)


class FailingStack(FakeStack):
    """FakeStack whose push fails on a frame holding 255 and whose finish
    fails for a negative reco radius, as a device or shape error would."""

    def push_frames(self, f):
        if np.any(np.asarray(f) == 255):
            raise RuntimeError("injected device error")
        super().push_frames(f)

    def finish(self, R):
        if R < 0:
            raise RuntimeError("injected reconstruction error")
        return super().finish(R)


class Producer:
    """Frames delivered by a producer thread: ``available()`` frames so far;
    ``stop_at`` freezes it there (a stalled producer)."""

    def __init__(self, frames, stop_at):
        self.frames, self.stop_at = frames, stop_at
        self.shape = frames.shape

    def __len__(self):
        return len(self.frames)

    def __getitem__(self, s):
        return self.frames[s]

    def available(self):
        return min(self.stop_at, len(self.frames))


def test_engine_isolates_failing_jobs():
    """A job whose push fails and one whose reconstruction fails end with an
    error; every other job completes with the result it has alone."""
    jobs = _jobs(14)
    jobs[3].frames = jobs[3].frames.copy()
    jobs[3].frames[len(jobs[3].frames) // 2, 0, 0] = 255  # fails in the middle of its frames
    jobs[7].reco_radius = -1.0
    eng = serve.Engine(max_active=4, workers=2, stack_factory=FailingStack)
    res, span = eng.run(jobs, realtime=False)
    by_id = {r.id: r for r in res}
    assert sorted(by_id) == list(range(14))
    assert by_id[3].error.startswith("push failed") and by_id[3].image is None
    assert by_id[7].error.startswith("finish failed") and by_id[7].nframes == len(jobs[7].frames)
    ok = [j for j in jobs if j.id not in (3, 7)]
    plain, _ = serve.run_plain(ok, realtime=False, stack_factory=FakeStack)
    for r in plain:
        assert by_id[r.id].error is None and np.array_equal(by_id[r.id].image, r.image)
    s = serve.summarize(res, span)
    assert s["jobs"] == 12 and s["failed"] == 2


def test_engine_stalled_producer_times_out():
    """A producer that stops after 16 of 40 frames fails its job after
    stall_timeout; the other jobs are served meanwhile."""
    jobs = _jobs(6)
    fr = np.random.default_rng(9).integers(0, 200, (40, 16, 16)).astype(np.uint8)
    jobs.append(serve.Job(99, Producer(fr, 16), 8, 6.0, chunk=8))
    eng = serve.Engine(max_active=8, workers=2, stack_factory=FakeStack, stall_timeout=0.05)
    res, _ = eng.run(jobs, realtime=False)
    by_id = {r.id: r for r in res}
    assert by_id[99].error.startswith("producer stalled") and by_id[99].nframes == 16
    assert all(by_id[j.id].error is None for j in jobs[:6])


def test_engine_cancel_while_streaming_and_waiting():
    """cancel() from another thread ends a job whose producer is stuck, and a
    job still waiting for admission; both report "cancelled"."""
    import threading

    jobs = _jobs(4)
    fr = np.random.default_rng(10).integers(0, 200, (40, 16, 16)).astype(np.uint8)
    jobs.append(serve.Job(50, Producer(fr, 8), 8, 6.0, chunk=8))     # never completes by itself
    jobs.append(serve.Job(51, fr, 8, 6.0, arrival=30.0, chunk=8))    # arrives far in the future
    eng = serve.Engine(max_active=8, workers=2, stack_factory=FakeStack)

    def stop():
        eng.cancel(50)
        eng.cancel(51)

    threading.Timer(0.05, stop).start()
    t = __import__("time").perf_counter()
    res, _ = eng.run(jobs, realtime=True)
    assert __import__("time").perf_counter() - t < 10.0
    by_id = {r.id: r for r in res}
    assert by_id[50].error == "cancelled" and by_id[50].nframes == 8
    assert by_id[51].error == "cancelled" and by_id[51].nframes == 0
    assert all(by_id[j.id].error is None for j in jobs[:4])


def test_engine_reco_mode_reaches_every_stack():
    made = []

    def factory(nc, nr, d):
        st = FakeStack(nc, nr, d)
        made.append(st)
        return st

    eng = serve.Engine(max_active=3, workers=2, stack_factory=factory, reco_mode="rings")
    res, _ = eng.run(_jobs(8), realtime=False)
    assert len(res) == 8 and made and all(getattr(st, "mode", None) == "rings" for st in made)
