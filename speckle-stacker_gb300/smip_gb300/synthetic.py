"""Seeded synthetic speckle stacks (workload generator for tests and benchmarks).

A frame is an object convolved with a short-exposure point-spread function
from a random Kolmogorov phase screen, plus Poisson photon noise, Gaussian
read noise, a bias level, clipping and quantisation to the frame's integer
type.  Every frame is generated from its own counter-based stream keyed by
``(seed, frame_index)``, so any chunking of a stack reproduces the same frames.

Workloads (all sizes are the reference's ``smip-cli`` parameters):

* ``binary``   -- two point sources 6 px apart, flux ratio 0.8 (u8 frames).
* ``extended`` -- a sum of Gaussian blobs with sigma 1-4 px and log-uniform
  fluxes (u16 frames); ``disk=True`` adds a smooth disk.

The telescope pupil is a disk of diameter N/2 pixels inside an N x N grid, so
the diffraction-limited core is Nyquist-sampled, and ``d_over_r0`` sets the
seeing (Fried parameter r0 = pupil diameter / d_over_r0).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

try:  # multi-threaded FFTs when scipy is present
    import scipy.fft as _sfft

    def _fft2(a):
        return _sfft.fft2(a, workers=-1)

    def _ifft2(a):
        return _sfft.ifft2(a, workers=-1)
except ImportError:  # pragma: no cover
    _fft2 = np.fft.fft2
    _ifft2 = np.fft.ifft2


@dataclass
class StackSpec:
    """One synthetic stack: its frames and the reconstruction parameters."""

    n: int                    # frame side (pixels)
    nframes: int
    kind: str = "binary"      # "binary" | "extended"
    dtype: str = "uint8"      # "uint8" | "uint16"
    d_over_r0: float = 10.0
    bdepth: int = 32          # smip-cli -b
    reco_radius: int = 64     # smip-cli -p
    seed: int = 1000
    nblobs: int = 20
    disk: bool = False
    peak_fraction: float = 0.6  # expected brightest pixel as a fraction of full scale
    extras: dict = field(default_factory=dict)

    @property
    def np_dtype(self):
        return np.dtype(self.dtype)


def config_spec(name: str, **kw) -> StackSpec:
    """The named workloads; keyword arguments override fields (e.g. nframes)."""
    if name == "binary128":      # 40 x 128^2 u8, D/r0 = 10, -b 32 -p 64
        s = StackSpec(n=128, nframes=40, kind="binary", dtype="uint8", d_over_r0=10.0,
                      bdepth=32, reco_radius=64, seed=1000)
    elif name == "extended256":  # 2000 x 256^2 u16, 20 blobs, D/r0 = 15, -b 32 -p 128
        s = StackSpec(n=256, nframes=2000, kind="extended", dtype="uint16", d_over_r0=15.0,
                      bdepth=32, reco_radius=128, seed=2000, nblobs=20)
    elif name == "extended512":  # 10000 x 512^2 u16, 200 blobs + disk, D/r0 = 25, -b 48 -p 200
        s = StackSpec(n=512, nframes=10000, kind="extended", dtype="uint16", d_over_r0=25.0,
                      bdepth=48, reco_radius=200, seed=5000, nblobs=200, disk=True)
    else:
        raise KeyError(name)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def _rng(seed: int, index: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(np.random.SeedSequence([int(seed), int(index)])))


def make_object(spec: StackSpec) -> np.ndarray:
    """Noise-free object (flux units, sums to 1), keyed by (seed, -1)."""
    n = spec.n
    obj = np.zeros((n, n), np.float64)
    c = n // 2
    if spec.kind == "binary":
        obj[c, c - 3] = 1.0
        obj[c, c + 3] = 0.8
    else:
        rng = _rng(spec.seed, 2**31 - 1)
        yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
        rad = n / 8.0
        for _ in range(spec.nblobs):
            r = rad * np.sqrt(rng.uniform())
            th = rng.uniform(0, 2 * np.pi)
            x0, y0 = c + r * np.cos(th), c + r * np.sin(th)
            sig = rng.uniform(1.0, 4.0)
            flux = np.exp(rng.uniform(np.log(0.1), np.log(1.0)))
            obj += flux / (2 * np.pi * sig * sig) * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * sig * sig))
        if spec.disk:
            rr = np.hypot(xx - c, yy - c)
            r0 = n / 6.0
            obj += 0.02 * 0.5 * (1 - np.tanh((rr - r0) / 2.0))
    return obj / obj.sum()


def _pupil(n: int) -> np.ndarray:
    yy, xx = np.mgrid[0:n, 0:n] - (n - 1) / 2.0
    return (np.hypot(xx, yy) <= n / 4.0).astype(np.float64)


def _phase_screen(rng: np.random.Generator, n: int, r0: float) -> np.ndarray:
    """Kolmogorov phase screen (radians) on a 2n x 2n grid, n x n corner returned."""
    m = 2 * n
    fx = np.fft.fftfreq(m)
    f = np.hypot(fx[None, :], fx[:, None])
    f[0, 0] = 1.0
    psd = 0.023 * r0 ** (-5.0 / 3.0) * f ** (-11.0 / 3.0)
    psd[0, 0] = 0.0
    c = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))) * np.sqrt(psd) / m
    scr = _fft2(c).real
    return scr[:n, :n]


def make_frame(spec: StackSpec, index: int, obj_ft: np.ndarray | None = None) -> np.ndarray:
    """Frame ``index`` of the stack as an (n, n) array of spec.dtype."""
    n = spec.n
    rng = _rng(spec.seed, index)
    if obj_ft is None:
        obj_ft = _fft2(make_object(spec))
    pupil = _pupil(n)
    r0 = (n / 2.0) / spec.d_over_r0
    phase = _phase_screen(rng, n, r0)
    field_ = _fft2(pupil * np.exp(1j * phase))
    psf = np.abs(field_) ** 2
    psf = np.fft.fftshift(psf / psf.sum())
    img = np.clip(_ifft2(_fft2(psf) * obj_ft).real, 0.0, None)
    img = np.fft.ifftshift(img)  # object centred in the frame
    full = float(np.iinfo(spec.np_dtype).max)
    # expected peak of a typical frame ~ peak_fraction * full scale
    scale = spec.peak_fraction * full / max(spec.extras.get("peak_norm", _peak_norm(spec)), 1e-30)
    bias = 0.04 * full
    counts = rng.poisson(img * scale).astype(np.float64) + bias + rng.normal(0.0, 2.0, (n, n))
    return np.clip(np.rint(counts), 0, full).astype(spec.np_dtype)


_PEAK_CACHE: dict = {}


def _peak_norm(spec: StackSpec) -> float:
    """Mean brightest-pixel value of a few noise-free frames (sets the exposure)."""
    key = (spec.n, spec.kind, spec.d_over_r0, spec.seed, spec.nblobs, spec.disk)
    if key not in _PEAK_CACHE:
        obj_ft = _fft2(make_object(spec))
        pupil = _pupil(spec.n)
        r0 = (spec.n / 2.0) / spec.d_over_r0
        peaks = []
        for i in range(4):
            rng = _rng(spec.seed + 7919, i)
            field_ = _fft2(pupil * np.exp(1j * _phase_screen(rng, spec.n, r0)))
            psf = np.abs(field_) ** 2
            psf = np.fft.fftshift(psf / psf.sum())
            peaks.append(np.clip(_ifft2(_fft2(psf) * obj_ft).real, 0, None).max())
        _PEAK_CACHE[key] = float(np.mean(peaks))
    return _PEAK_CACHE[key]


def make_stack(spec: StackSpec, start: int = 0, count: int | None = None, procs: int = 1) -> np.ndarray:
    """Frames [start, start+count) as an (count, n, n) array.

    procs > 1 generates chunks in a pool of fresh ("spawn") processes, which
    is safe after CUDA has been initialised in this process; the frames are
    the same for any chunking."""
    count = spec.nframes - start if count is None else count
    if procs > 1 and count >= 2 * procs:
        import multiprocessing as mp

        chunk = (count + procs - 1) // procs
        jobs = [(spec, start + s, min(chunk, count - s)) for s in range(0, count, chunk)]
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            return np.concatenate(pool.starmap(make_stack, jobs))
    obj_ft = _fft2(make_object(spec))
    out = np.empty((count, spec.n, spec.n), spec.np_dtype)
    for k in range(count):
        out[k] = make_frame(spec, start + k, obj_ft)
    return out
