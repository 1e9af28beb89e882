"""Batched and served execution of many speckle-masking jobs on one GPU.

The reference runs one job per ``smip-cli`` process (smip-cli/main.cpp:232-376);
a job's accumulators are additive and independent of every other job's.  Here
many jobs share one device:

* every job owns a device-resident stack (packed bispectrum + compensation,
  power spectrum, shift-and-add sum, reference frame) running on its own CUDA
  stream, so the kernels of different jobs overlap on the GPU;
* **continuous batching**: a request loop admits arriving jobs while slots and
  bispectrum memory are free (admission is by bispectrum bytes under a budget),
  streams every admitted job's frames in chunks, round robin, and hands a job
  whose frames are all in to a worker thread for phase recovery and the final
  image, while the loop keeps feeding the others;
* stacks are pooled by shape and reset between jobs, so the loop allocates no
  device memory after warm-up;
* a job fails alone: an error while its frames are pushed or while it is
  reconstructed, a producer that delivers no frames for ``stall_timeout``
  seconds, or ``Engine.cancel`` gives that job a result with ``error`` set
  and its bytes back to the budget, while the other jobs go on.

``run_plain`` is the single-job path (one job at a time, in arrival order)
that the served numbers are compared with.  A job's results do not depend on
what else runs: each stack batches its own frames the same way alone and in a
mix, so results are identical, which ``tests/test_serve.py`` checks.
"""
from __future__ import annotations

import concurrent.futures as cf
import threading
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np


class FrameRing:
    """``count`` frames read cyclically from a frame bank starting at
    ``offset`` (no copy; the bank may be page-locked host memory)."""

    def __init__(self, bank: np.ndarray, offset: int, count: int):
        self.bank, self.offset, self.count = bank, int(offset), int(count)
        self.shape = (self.count,) + bank.shape[1:]

    def __len__(self):
        return self.count

    def parts(self, pos: int, k: int):
        """Contiguous pieces holding frames [pos, pos + k)."""
        out, n = [], len(self.bank)
        while k > 0:
            i = (self.offset + pos) % n
            m = min(k, n - i)
            out.append(self.bank[i:i + m])
            pos, k = pos + m, k - m
        return out

    def materialize(self) -> np.ndarray:
        return np.concatenate(self.parts(0, self.count))


@dataclass
class Job:
    """One reconstruction request: frames plus smip-cli's -b and -p."""

    id: int
    frames: object              # [nframes][rows][cols] array (u8/u16/f32/f64) or a FrameRing
    bdepth: int
    reco_radius: float
    arrival: float = 0.0        # seconds after the run starts
    chunk: int = 32             # frames delivered per push

    @property
    def shape(self) -> Tuple[int, int, int]:
        return (self.frames.shape[2], self.frames.shape[1], self.bdepth)

    def available(self) -> int:
        """Frames the producer has delivered so far: a frame source with an
        ``available()`` method (frames still arriving) reports it, an array
        or FrameRing holds all of them."""
        f = getattr(self.frames, "available", None)
        return int(f()) if callable(f) else len(self.frames)

    def parts(self, pos: int, k: int):
        if isinstance(self.frames, FrameRing):
            return self.frames.parts(pos, k)
        return [self.frames[pos:pos + k]]


@dataclass
class JobResult:
    id: int
    nframes: int
    arrival: float
    admitted: float
    done: float
    image: Optional[np.ndarray] = field(repr=False)
    phases: Optional[np.ndarray] = field(repr=False)
    flags: Optional[np.ndarray] = field(repr=False)
    consistency: Optional[np.ndarray] = field(repr=False)
    shifts: Optional[np.ndarray] = field(repr=False)
    error: Optional[str] = None  # set (arrays None) when the job failed or was cancelled

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def bispectrum_bytes(ncols: int, nrows: int, bdepth: int) -> int:
    """Device bytes of one job's bispectrum: the packed accumulator, its Kahan
    compensation and the normalised copy (complex<float> each)."""
    d = (bdepth // 2) * 2
    base = (ncols // 2 + 1) * (nrows + 1) * (d // 2 + 1) * (d + 1)
    return 3 * 8 * base


def summarize(results: List[JobResult], makespan: float) -> dict:
    """Throughput and latency of the jobs that completed; failed or cancelled
    jobs are counted apart."""
    ok = [r for r in results if r.error is None]
    lat = np.array([r.latency for r in ok] or [0.0]) * 1e3
    frames = sum(r.nframes for r in ok)
    out = {"jobs": len(ok), "frames": frames, "seconds": makespan, "frames_per_s": frames / makespan,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
    if len(ok) != len(results):
        out["failed"] = len(results) - len(ok)
    return out


class Engine:
    """Continuous-batching request loop over a pool of device-resident stacks.

    budget_bytes: admission budget in bispectrum bytes (``bispectrum_bytes``).
    max_active: jobs in flight at once (streaming or reconstructing).
    workers: threads that run phase recovery + the final image.
    stack_factory: (ncols, nrows, bdepth) -> stack; defaults to smip_gb300.Stack.
    graph: the last batches of the jobs whose frames are all in after a round
        run together (smip_gb300.batch_launch: their bispectrum work as one
        persistent launch from a captured CUDA graph) before their
        reconstructions start, instead of one flush per job.  The jobs of a
        round go in groups of ``graph_group`` (largest frames first), each
        group's reconstructions submitted right after its launch; while
        reconstructions are in flight a launch leaves ``graph_reserve`` SMs
        out of its grid, so that they run beside it.
    stall_timeout: seconds a streaming job may go without new frames from its
        producer before it fails (None: wait for ever).
    reco_mode: "spiral" (the reference's phase recovery, default) or "rings"
        (the opt-in ring-parallel estimator, Stack.set_reco_mode).
    chunks_per_round: a streaming job pushes up to this many of its delivered
        chunks per round (whole chunks), so that the request loop's host
        work per frame stays small when many jobs stream at once.
    """

    def __init__(self, device: int = 0, budget_bytes: float = 120e9, max_active: int = 64, workers: int = 32,
                 stack_factory: Optional[Callable] = None, graph: bool = False,
                 batch_launch: Optional[Callable] = None, stall_timeout: Optional[float] = None,
                 reco_mode: str = "spiral", chunks_per_round: int = 8, graph_group: int = 8,
                 graph_reserve: int = 16):
        if stack_factory is None:
            from smip_gb300 import Stack

            def stack_factory(nc, nr, d):
                return Stack(nc, nr, d, device=device)
        if graph and batch_launch is None:
            from smip_gb300 import batch_launch
        self.factory = stack_factory
        self.graph = bool(graph)
        self.batch_launch = batch_launch
        self.budget = float(budget_bytes)
        self.max_active = int(max_active)
        self.workers = int(workers)
        self.stall_timeout = stall_timeout
        self.reco_mode = reco_mode
        self.chunks_per_round = max(1, int(chunks_per_round))
        self.graph_group = max(1, int(graph_group))
        self.graph_reserve = max(0, int(graph_reserve))
        self.pool: Dict[Tuple[int, int, int], list] = {}
        self.peak_bytes = 0.0
        self.peak_active = 0
        self._cancel_lock = threading.Lock()
        self._cancelled: set = set()

    def cancel(self, job_id: int):
        """Cancels a job that is waiting or still streaming (callable from any
        thread while ``run`` serves).  It ends with error "cancelled" and its
        stack goes back to the pool; a job already being reconstructed
        completes normally."""
        with self._cancel_lock:
            self._cancelled.add(job_id)

    def _is_cancelled(self, job_id: int) -> bool:
        with self._cancel_lock:
            return job_id in self._cancelled

    def prewarm(self, shapes, count: int = 1, reco_radius=None):
        """Creates ``count`` pooled stacks per (ncols, nrows, bdepth) shape, so
        that no device allocation happens while jobs are served.
        reco_radius (a number, or a function of the shape): the radius the
        jobs of a shape reconstruct with; the stacks' reconstruction buffers
        are then allocated here as well."""
        for s in shapes:
            lst = self.pool.setdefault(tuple(s), [])
            while len(lst) < count:
                lst.append(self.factory(*s))
            if reco_radius is not None:
                r = reco_radius(tuple(s)) if callable(reco_radius) else reco_radius
                for st in lst:
                    prep = getattr(st, "prepare_reco", None)
                    if callable(prep):
                        prep(r)

    def _acquire(self, shape):
        lst = self.pool.setdefault(shape, [])
        st = lst.pop() if lst else self.factory(*shape)
        setter = getattr(st, "set_reco_mode", None)
        if callable(setter):  # pooled stacks may come from a run in the other mode
            setter(self.reco_mode)
        return st

    def _release(self, shape, st):
        try:
            st.reset()
        except Exception:  # a stack that cannot be reset is not reused
            self._discard(st)
            return
        self.pool.setdefault(shape, []).append(st)

    @staticmethod
    def _finish(job: Job, st, t0: float, admitted: float) -> JobResult:
        img, ph, fl, cs = st.finish(job.reco_radius)
        sh = st.shifts()
        return JobResult(job.id, len(job.frames), job.arrival, admitted, time.perf_counter() - t0, img, ph, fl, cs, sh)

    @staticmethod
    def _failed(job: Job, t0: float, admitted: float, nframes: int, why: str) -> JobResult:
        return JobResult(job.id, nframes, job.arrival, admitted, time.perf_counter() - t0, None, None, None, None,
                         None, error=why)

    @staticmethod
    def _discard(st):
        """A stack whose job failed on a device call is not reused."""
        close = getattr(st, "close", None)
        if callable(close):
            try:
                close()
            except Exception:  # the failure is already reported for the job
                pass

    def run(self, jobs: List[Job], realtime: bool = True) -> Tuple[List[JobResult], float]:
        """Serves ``jobs``; with ``realtime`` a job is only visible from its
        arrival time on, otherwise all are queued at once (batched mode).
        Returns (results in completion order, makespan in seconds)."""
        waiting = sorted(jobs, key=lambda j: (j.arrival, j.id))
        active: list = []          # [job, stack, frames pushed, admitted time, bytes, time of last frames]
        running: dict = {}         # future -> (job, stack, bytes, admitted time)
        results: List[JobResult] = []
        used = 0.0
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=self.workers) as ex:
            while waiting or active or running:
                now = time.perf_counter() - t0
                for job in [j for j in waiting if self._is_cancelled(j.id)]:
                    waiting.remove(job)
                    results.append(self._failed(job, t0, now, 0, "cancelled"))
                # admission: FIFO, by slots and bispectrum bytes
                while waiting and (not realtime or waiting[0].arrival <= now) \
                        and len(active) + len(running) < self.max_active:
                    job = waiting[0]
                    need = bispectrum_bytes(*job.shape)
                    if used + need > self.budget and (active or running):
                        break
                    waiting.pop(0)
                    used += need
                    active.append([job, self._acquire(job.shape), 0, now, need, now])
                self.peak_bytes = max(self.peak_bytes, used)
                self.peak_active = max(self.peak_active, len(active) + len(running))
                # the delivered chunks of every streaming job, round robin
                pushed = False
                ready = []
                for entry in list(active):
                    job, st, pos = entry[0], entry[1], entry[2]
                    why = None
                    if self._is_cancelled(job.id):
                        why = "cancelled"
                    else:
                        avail = min(job.available(), len(job.frames)) - pos
                        k = min(job.chunk * self.chunks_per_round, avail)
                        if k < avail:  # whole chunks only, unless it is the job's last piece
                            k -= k % job.chunk
                        if k > 0:
                            try:
                                for part in job.parts(pos, k):
                                    st.push_frames(part)
                            except Exception as e:  # this job's frames or device call failed
                                active.remove(entry)
                                used -= entry[4]
                                self._discard(st)
                                results.append(self._failed(job, t0, entry[3], pos, f"push failed: {e}"))
                                continue
                            entry[2] = pos + k
                            entry[5] = now
                            pushed = True
                        elif self.stall_timeout is not None and now - entry[5] > self.stall_timeout:
                            why = f"producer stalled: no frames for {self.stall_timeout:g} s after frame {pos}"
                    if why is not None:
                        active.remove(entry)
                        used -= entry[4]
                        self._release(job.shape, st)
                        results.append(self._failed(job, t0, entry[3], entry[2], why))
                    elif entry[2] == len(job.frames):
                        active.remove(entry)
                        ready.append(entry)
                groups = [ready]
                if self.graph and ready:  # longest reconstructions (largest frames) first
                    ready.sort(key=lambda e: -e[0].shape[0] * e[0].shape[1])
                    groups = [ready[i:i + self.graph_group] for i in range(0, len(ready), self.graph_group)]
                for grp in groups:
                    if self.graph:
                        self.batch_launch([e[1] for e in grp], reserve_sms=self.graph_reserve if running else 0)
                    for entry in grp:
                        fut = ex.submit(self._finish, entry[0], entry[1], t0, entry[3])
                        running[fut] = (entry[0], entry[1], entry[4], entry[3])
                # completions
                done = [f for f in running if f.done()]
                for f in done:
                    job, st, need, admitted = running.pop(f)
                    used -= need
                    try:
                        results.append(f.result())
                    except Exception as e:  # reconstruction failed: report it, drop the stack
                        self._discard(st)
                        results.append(self._failed(job, t0, admitted, len(job.frames), f"finish failed: {e}"))
                        continue
                    self._release(job.shape, st)
                if not pushed and not done:
                    if running:
                        cf.wait(list(running), timeout=0.002, return_when=cf.FIRST_COMPLETED)
                    elif active:
                        time.sleep(0.001)  # every streaming job waits for its producer
                    elif waiting:
                        time.sleep(max(0.0, min(0.002, waiting[0].arrival - (time.perf_counter() - t0))))
        return results, time.perf_counter() - t0


def run_plain(jobs: List[Job], device: int = 0, realtime: bool = True,
              stack_factory: Optional[Callable] = None) -> Tuple[List[JobResult], float]:
    """The single-job path: one job at a time in arrival order, each pushed
    completely and reconstructed before the next starts (one pooled stack per
    shape)."""
    if stack_factory is None:
        from smip_gb300 import Stack

        def stack_factory(nc, nr, d):
            return Stack(nc, nr, d, device=device)
    pool: dict = {}
    results = []
    t0 = time.perf_counter()
    for job in sorted(jobs, key=lambda j: (j.arrival, j.id)):
        if realtime:
            wait = job.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        st = pool.get(job.shape)
        if st is None:
            st = pool[job.shape] = stack_factory(*job.shape)
        admitted = time.perf_counter() - t0
        for pos in range(0, len(job.frames), job.chunk):
            for part in job.parts(pos, min(job.chunk, len(job.frames) - pos)):
                st.push_frames(part)
        results.append(Engine._finish(job, st, t0, admitted))
        st.reset()
    return results, time.perf_counter() - t0


# ------------------------------------------------------------- workloads
def _bank(n: int, kind: str, count: int, seed: int, procs: int = 1):
    from smip_gb300 import synthetic as S

    spec = S.StackSpec(n=n, nframes=count, kind=kind, dtype="uint8" if kind == "binary" else "uint16",
                       d_over_r0=10.0 if kind == "binary" else 15.0, seed=seed)
    if procs <= 1:
        return S.make_stack(spec, 0, count)
    import multiprocessing as mp

    step = (count + procs - 1) // procs
    parts = [(spec, s, min(step, count - s)) for s in range(0, count, step)]
    with mp.get_context("spawn").Pool(procs) as pool:
        return np.concatenate(pool.starmap(S.make_stack, parts))


def depth_for(n: int) -> int:
    """Bispectrum depth scaled per stack size: 16 at 64^2, 24 at 128^2, 32 at 256^2."""
    return {64: 16, 128: 24, 256: 32}[n]


def make_jobs(njobs: int, sizes=(64, 128, 256), counts=(50, 1000), rate: Optional[float] = None,
              seed: int = 3000, bank_frames: int = 256, procs: int = 1, chunk: int = 32,
              pin: bool = False) -> List[Job]:
    """Uneven jobs: frame size drawn from ``sizes``, frame count uniform in
    ``counts``, binary or extended objects 50/50, depth scaled per size and
    reco radius 2 x depth (smip-cli's default ratio).  A job's frames are a
    cyclic run through a seeded per-(size, kind) frame bank.  ``rate``:
    Poisson arrivals (jobs/s), else all arrive at t = 0.  ``pin``: banks in
    page-locked host memory (torch), so pushes are asynchronous."""
    rng = np.random.default_rng(seed)
    plan = []
    t = 0.0
    for i in range(njobs):
        n = int(rng.choice(sizes))
        kind = "binary" if rng.uniform() < 0.5 else "extended"
        cnt = int(rng.integers(counts[0], counts[1] + 1))
        off = int(rng.integers(0, bank_frames))
        if rate:
            t += float(rng.exponential(1.0 / rate))
        plan.append((i, n, kind, cnt, off, t if rate else 0.0))
    banks = {}
    for key in sorted({(n, kind) for _, n, kind, _, _, _ in plan}):
        n, kind = key
        b = _bank(n, kind, bank_frames, seed + 7 * n + (kind == "extended"), procs)
        if pin:
            import torch

            tt = torch.from_numpy(np.ascontiguousarray(b)).pin_memory()
            banks[key] = (tt.numpy(), tt)  # the tensor keeps the page-locked memory alive
        else:
            banks[key] = (b, None)
    jobs = []
    for i, n, kind, cnt, off, arr in plan:
        d = depth_for(n)
        job = Job(i, FrameRing(banks[(n, kind)][0], off, cnt), d, 2.0 * d, arrival=arr, chunk=chunk)
        job.bank_owner = banks[(n, kind)][1]
        jobs.append(job)
    return jobs


def pin_banks(jobs: List[Job]):
    """Moves the jobs' frame banks into page-locked host memory (torch), so
    pushes from them are asynchronous; returns the owners to keep alive."""
    import torch

    pinned, owners = {}, []
    for job in jobs:
        fr = job.frames
        if not isinstance(fr, FrameRing):
            continue
        key = id(fr.bank)
        if key not in pinned:
            tt = torch.from_numpy(np.ascontiguousarray(fr.bank)).pin_memory()
            pinned[key] = tt.numpy()
            owners.append(tt)
        fr.bank = pinned[key]
    return owners


def compare_results(a: List[JobResult], b: List[JobResult]) -> bool:
    """True when every job has bit-identical shifts, flags, phases and image."""
    bb = {r.id: r for r in b}
    return all(np.array_equal(r.shifts, bb[r.id].shifts) and np.array_equal(r.flags, bb[r.id].flags)
               and np.array_equal(r.phases, bb[r.id].phases) and np.array_equal(r.image, bb[r.id].image)
               for r in a)
