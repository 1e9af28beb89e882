"""Python host binding of the GB300 SMIP engine (libsmip_gpu.so via ctypes).

The names mirror hangeza/speckle-stacker's C++ API for the hot path:

* :class:`Stack` -- the per-job accumulators of smip-cli/main.cpp:232-312
  (bispectrum + Kahan compensation, power spectrum, shift-and-add sum) with
  ``push_frames`` (main.cpp:281-306), ``accumulate_from_fft``
  (include/bispectrum.h:82-83), ``reconstruct_phases`` (phasereco.h:16-19) and
  ``finish`` (main.cpp:318-376).
* :func:`reconstruct_phases`, :func:`next_reco_index`, :class:`CrossCorrelation`,
  :func:`hann` -- the reference's free functions and classes.

Status codes from the C ABI are raised as the Python counterparts of the
reference's exception types.  There is no CPU fallback: the first call into
the library raises ImportError when libsmip_gpu.so has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libsmip_gpu.so")

U8, U16, F32, F64 = 0, 1, 2, 3
_DTYPES = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16, np.dtype(np.float32): F32, np.dtype(np.float64): F64}


# ---------------------------------------------------------------- exceptions
class SmipError(Exception):
    """Base class of errors reported by libsmip_gpu."""


class InvalidArgument(SmipError, ValueError):       # std::invalid_argument
    pass


class OutOfRange(SmipError, IndexError):            # std::out_of_range
    pass


class RuntimeFailure(SmipError, RuntimeError):      # std::runtime_error
    pass


class DomainError(SmipError, ValueError):           # std::domain_error
    pass


class BadFunctionCall(SmipError, RuntimeError):     # std::bad_function_call
    pass


class NoMemory(SmipError, MemoryError):
    pass


class CudaError(SmipError, RuntimeError):
    pass


class DeviceTimeout(SmipError, TimeoutError):
    pass


class Unsupported(SmipError, NotImplementedError):
    pass


_ERRORS = {1: InvalidArgument, 2: OutOfRange, 3: RuntimeFailure, 4: DomainError, 5: BadFunctionCall,
           6: NoMemory, 7: CudaError, 8: DeviceTimeout, 9: Unsupported}


def build() -> None:
    """Compile libsmip_gpu.so for sm_103a (make -j in the package directory)."""
    subprocess.run(["make", "-s", "-C", PKG_DIR, f"-j{min(8, os.cpu_count() or 1)}"], check=True)


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libsmip_gpu.so not built ({LIB_PATH}); run smip_gb300.build() / __graft_entry__.build()")
    lib = C.CDLL(LIB_PATH)
    vp, dp, fp, ip, lp, ubp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int), \
        C.POINTER(C.c_long), C.POINTER(C.c_ubyte)
    sig = {
        "smip_last_error": ([], C.c_char_p),
        "smip_version": ([ip, ip, ip], C.c_int),
        "smip_stack_create": ([C.POINTER(vp), C.c_int, C.c_long, C.c_long, C.c_long, vp, C.c_long], C.c_int),
        "smip_stack_destroy": ([vp], C.c_int),
        "smip_stack_push_frames": ([vp, vp, C.c_int, C.c_long, C.c_long, C.c_int], C.c_int),
        "smip_stack_accumulate_fft": ([vp, vp, C.c_long, C.c_int], C.c_int),
        "smip_stack_flush": ([vp], C.c_int),
        "smip_stack_sync": ([vp], C.c_int),
        "smip_stack_frame_count": ([vp, lp], C.c_int),
        "smip_stack_bispectrum_size": ([vp, lp], C.c_int),
        "smip_stack_shifts": ([vp, ip, C.c_long, C.c_long], C.c_int),
        "smip_stack_sum": ([vp, dp], C.c_int),
        "smip_stack_power": ([vp, dp], C.c_int),
        "smip_stack_bispectrum": ([vp, fp], C.c_int),
        "smip_stack_reconstruct": ([vp, C.c_double, dp, ubp, dp], C.c_int),
        "smip_stack_finish": ([vp, C.c_double, dp, dp, ubp, dp], C.c_int),
        "smip_stack_prepare_reco": ([vp, C.c_double], C.c_int),
        "smip_stack_merge": ([vp, vp], C.c_int),
        "smip_stack_set_kernel_config": ([vp, C.c_int, C.c_int], C.c_int),
        "smip_batch_launch": ([C.POINTER(vp), C.c_long], C.c_int),
        "smip_batch_launch_reserve": ([C.POINTER(vp), C.c_long, C.c_int], C.c_int),
        "smip_diag_bounded_wait": ([C.c_int, C.c_double], C.c_int),
        "smip_stack_set_bispectrum": ([vp, fp, C.c_long], C.c_int),
        "smip_stack_save_state": ([vp, C.c_char_p], C.c_int),
        "smip_stack_load_state": ([vp, C.c_char_p], C.c_int),
        "smip_stack_share_reference": ([vp, vp], C.c_int),
        "smip_stack_save_bispectrum": ([vp, C.c_char_p], C.c_int),
        "smip_stack_load_bispectrum": ([vp, C.c_char_p, C.c_long], C.c_int),
        "smip_reconstruct_phases": ([C.c_int, fp, C.c_long, C.c_long, C.c_long, C.c_double, dp, ubp, dp], C.c_int),
        "smip_next_reco_index": ([dp, dp, ip, ip], C.c_int),
        "smip_reco_visits": ([C.c_double, ip, C.c_long, lp], C.c_int),
        "smip_xcorr_displacement": ([C.c_int, dp, dp, C.c_long, C.c_long, ip, ip, dp], C.c_int),
        "smip_hann": ([C.c_int, dp, C.c_long, C.c_long, C.c_double], C.c_int),
        "smip_shifted": ([C.c_int, dp, dp, C.c_long, C.c_long, C.c_int, C.c_int], C.c_int),
        "smip_bispec_offsets": ([C.c_int, C.c_long, C.c_long, C.c_long, ip, C.c_long,
                                 C.POINTER(C.c_longlong), ip], C.c_int),
        "smip_xcorr_displacement_noalloc": ([vp, vp, C.c_long, C.c_long, vp, vp], C.c_int),
        "smip_stack_reset": ([vp], C.c_int),
        "smip_stack_set_reco_mode": ([vp, C.c_int], C.c_int),
        "smip_stack_set_timing": ([vp, C.c_int], C.c_int),
        "smip_stack_kernel_time": ([vp, dp, lp, dp], C.c_int),
        "smip_kernel_launches": ([], C.c_longlong),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


_lib_handle = None


def _L():
    """The loaded library (loaded on first use; ImportError if it is not built)."""
    global _lib_handle
    if _lib_handle is None:
        _lib_handle = _load()
    return _lib_handle


def _check(rc: int) -> None:
    if rc != 0:
        msg = _L().smip_last_error().decode(errors="replace")
        raise _ERRORS.get(rc, SmipError)(msg)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def version():
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    _check(_L().smip_version(C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def batch_launch(stacks, reserve_sms: int = 0) -> None:
    """Runs the pending frame batches of ``stacks``: each stack's per-frame
    kernels on its own stream, then the bispectrum work of all of them as one
    persistent launch (a CUDA graph captured once per grid size); stacks
    without pending frames are skipped.  Later calls on each stack are ordered
    after it.  reserve_sms: streaming multiprocessors left out of the
    persistent grid, for the phase recoveries of earlier stacks."""
    stacks = list(stacks)
    arr = (C.c_void_p * max(1, len(stacks)))(*[st._h.value for st in stacks])
    _check(_L().smip_batch_launch_reserve(arr, len(stacks), int(reserve_sms)))


def diag_bounded_wait(device: int = 0, timeout_s: float = 0.05) -> None:
    """Runs a kernel whose bounded waits can never be satisfied; raises
    DeviceTimeout, as any call does after an expired device wait."""
    _check(_L().smip_diag_bounded_wait(device, float(timeout_s)))


def kernel_launches() -> int:
    """Kernels libsmip_gpu has launched in this process."""
    return int(_L().smip_kernel_launches())


def bispec_base_size(ncols, nrows, depth):
    """(ncols/2+1)(nrows+1)(d/2+1)(d+1), d = depth rounded down to even (bispectrum.h:213-220)."""
    d = (depth // 2) * 2
    return ((ncols // 2) * 2 + 1 - (ncols // 2)) * ((nrows // 2) * 2 + 1) * (d + 1 - d // 2) * (d + 1)


# ------------------------------------------------------------------ Stack
class Stack:
    """Device-resident speckle-masking accumulators for one stack of frames."""

    def __init__(self, ncols: int, nrows: int, bdepth: int, device: int = 0, stream: int | None = None,
                 batch_frames=0, dtype=np.uint16):
        """batch_frames: frames per accumulation batch; 0 = library default,
        "auto" = the autotuner's cached best for this device and shape (tuned
        on first use, smip_gb300.autotune); dtype only informs "auto"."""
        tuned = None
        if batch_frames == "auto":
            from smip_gb300 import autotune

            tuned = autotune.best_config(ncols, nrows, bdepth, dtype, device)
            batch_frames = tuned["batch_frames"]
        h = C.c_void_p()
        _check(_L().smip_stack_create(C.byref(h), device, ncols, nrows, bdepth,
                                      C.c_void_p(stream) if stream else None, batch_frames))
        self._h = h
        self.ncols, self.nrows, self.bdepth, self.device = ncols, nrows, bdepth, device
        if tuned is not None:
            self.set_kernel_config(tuned["variant"], tuned["min_part"])

    def close(self):
        if getattr(self, "_h", None):
            _L().smip_stack_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- input --------------------------------------------------------------
    def push_frames(self, frames, on_device: bool = False):
        """frames: numpy array (n, nrows, ncols) or (nrows, ncols) of u8/u16/f32/f64,
        or a CUDA torch tensor of those types (on_device inferred)."""
        if hasattr(frames, "data_ptr"):  # torch tensor
            t = frames
            if t.dim() == 2:
                t = t.unsqueeze(0)
            tmap = {"torch.uint8": U8, "torch.uint16": U16, "torch.float32": F32, "torch.float64": F64}
            dt = tmap.get(str(t.dtype))
            if dt is None:
                raise InvalidArgument(f"unsupported frame dtype {t.dtype}")
            if not t.is_contiguous():
                t = t.contiguous()
            n = t.shape[0]
            _check(_L().smip_stack_push_frames(self._h, C.c_void_p(t.data_ptr()), dt, n, 0, 1 if t.is_cuda else 0))
            return
        a = np.asarray(frames)
        if a.ndim == 2:
            a = a[None]
        a = np.ascontiguousarray(a)
        if a.dtype not in _DTYPES:
            raise InvalidArgument(f"unsupported frame dtype {a.dtype}")
        if a.shape[1:] != (self.nrows, self.ncols):
            raise InvalidArgument("Matrix dimensions must match")
        _check(_L().smip_stack_push_frames(self._h, a.ctypes.data, _DTYPES[a.dtype], a.shape[0], 0,
                                           1 if on_device else 0))

    def accumulate_from_fft(self, spectra):
        """Bispectrum::accumulate_from_fft for FFT-order complex<double> spectra."""
        a = np.ascontiguousarray(spectra, dtype=np.complex128)
        if a.ndim == 2:
            a = a[None]
        _check(_L().smip_stack_accumulate_fft(self._h, a.ctypes.data, a.shape[0], 0))

    def set_kernel_config(self, variant: int = 0, min_part: int = 0):
        """Bispectrum kernel tuning: variant 0 (four frames per ring stage) or
        1 (two); min_part: fewest frames per split part of a last-wave tile
        (0 = 8).  The autotuner picks both ("auto" batch_frames)."""
        _check(_L().smip_stack_set_kernel_config(self._h, int(variant), int(min_part)))

    def prepare_reco(self, reco_radius: float):
        """Allocates the reconstruction's buffers and visit tables for
        reco_radius now, so that finish() with that radius allocates nothing
        (a serving loop prepares its pooled stacks)."""
        _check(_L().smip_stack_prepare_reco(self._h, float(reco_radius)))

    def set_reco_mode(self, mode="spiral"):
        """Phase-recovery estimator: "spiral" (default, the reference's walk)
        or "rings" (each turn of the spiral in parallel from earlier turns
        only: faster, not the reference's estimator)."""
        m = {"spiral": 0, "rings": 1}.get(mode, mode)
        _check(_L().smip_stack_set_reco_mode(self._h, int(m)))

    def reset(self):
        """Zero the accumulators for a new job (device buffers are kept)."""
        _check(_L().smip_stack_reset(self._h))

    def set_timing(self, on: bool = True):
        """Record CUDA events around each bispectrum-kernel launch."""
        _check(_L().smip_stack_set_timing(self._h, 1 if on else 0))

    def kernel_time(self):
        """(bispectrum kernel ms, launches, frames) since the last call."""
        ms, n, fr = C.c_double(), C.c_long(), C.c_double()
        _check(_L().smip_stack_kernel_time(self._h, C.byref(ms), C.byref(n), C.byref(fr)))
        return ms.value, n.value, fr.value

    def flush(self):
        _check(_L().smip_stack_flush(self._h))

    def sync(self):
        _check(_L().smip_stack_sync(self._h))

    # -- results ------------------------------------------------------------
    @property
    def nframes(self) -> int:
        n = C.c_long()
        _check(_L().smip_stack_frame_count(self._h, C.byref(n)))
        return n.value

    @property
    def base_size(self) -> int:
        n = C.c_long()
        _check(_L().smip_stack_bispectrum_size(self._h, C.byref(n)))
        return n.value

    def shifts(self, first: int = 0, count: int | None = None):
        count = self.nframes - first if count is None else count
        out = np.zeros((count, 2), np.int32)
        _check(_L().smip_stack_shifts(self._h, _p(out, C.c_int), first, count))
        return out

    def sum(self):
        out = np.zeros((self.nrows, self.ncols), np.float64)
        _check(_L().smip_stack_sum(self._h, _p(out, C.c_double)))
        return out

    def power(self):
        out = np.zeros((self.nrows, self.ncols), np.float64)
        _check(_L().smip_stack_power(self._h, _p(out, C.c_double)))
        return out

    def bispectrum(self):
        out = np.zeros(self.base_size, np.complex64)
        _check(_L().smip_stack_bispectrum(self._h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def reconstruct_phases(self, reco_radius: float):
        n = self.nrows * self.ncols
        ph = np.zeros(n, np.complex128)
        fl = np.zeros(n, np.uint8)
        cs = np.zeros(n, np.float64)
        _check(_L().smip_stack_reconstruct(self._h, float(reco_radius), ph.ctypes.data_as(C.POINTER(C.c_double)),
                                           _p(fl, C.c_ubyte), _p(cs, C.c_double)))
        s = (self.nrows, self.ncols)
        return ph.reshape(s), fl.reshape(s), cs.reshape(s)

    def finish(self, reco_radius: float):
        """(image, phases, flags, consistency) of main.cpp:318-376."""
        n = self.nrows * self.ncols
        img = np.zeros(n, np.complex128)
        ph = np.zeros(n, np.complex128)
        fl = np.zeros(n, np.uint8)
        cs = np.zeros(n, np.float64)
        dp = C.POINTER(C.c_double)
        _check(_L().smip_stack_finish(self._h, float(reco_radius), img.ctypes.data_as(dp), ph.ctypes.data_as(dp),
                                      _p(fl, C.c_ubyte), _p(cs, C.c_double)))
        s = (self.nrows, self.ncols)
        return img.reshape(s), ph.reshape(s), fl.reshape(s), cs.reshape(s)

    def merge(self, other: "Stack"):
        _check(_L().smip_stack_merge(self._h, other._h))

    def share_reference(self, other: "Stack"):
        """Make ``other`` correlate its frames against this stack's frame 0."""
        _check(_L().smip_stack_share_reference(self._h, other._h))

    def save_bispectrum(self, path: str):
        _check(_L().smip_stack_save_bispectrum(self._h, path.encode()))

    def load_bispectrum(self, path: str, nframes: int = 0):
        """Bispectrum::read_from_file (bispectrum.h:432-462) into this empty
        stack: the accumulator resumes as the file's normalised bispectrum x
        nframes (0 = 1); reconstruct_phases and accumulate_from_fft work on it."""
        _check(_L().smip_stack_load_bispectrum(self._h, path.encode(), int(nframes)))

    def save_state(self, path: str):
        """Whole-stack checkpoint (after a flush): accumulators, shifts and the
        reference frame; load_state on an empty stack of the same shape resumes."""
        _check(_L().smip_stack_save_state(self._h, path.encode()))

    def load_state(self, path: str):
        _check(_L().smip_stack_load_state(self._h, path.encode()))

    def set_bispectrum(self, bispec, nframes: int = 0):
        """load_bispectrum from memory: a complex64 array of base_size, the
        packed normalised bispectrum (what bispectrum() returns)."""
        b = np.ascontiguousarray(bispec, np.complex64).ravel()
        if b.size != self.base_size:
            raise InvalidArgument(f"bispectrum has {b.size} elements, the stack {self.base_size}")
        _check(_L().smip_stack_set_bispectrum(self._h, b.ctypes.data_as(C.POINTER(C.c_float)), int(nframes)))


# ------------------------------------------------------- free functions
def reconstruct_phases(bispec, xsize: int, ysize: int, bdepth: int, reco_radius: float, device: int = 0):
    """reconstruct_phases<complex_t, complex<float>> on a packed complex64 bispectrum.
    Returns (phases complex128 (ysize, xsize), flags uint8, consistency float64)."""
    b = np.ascontiguousarray(bispec, np.complex64)
    if b.size != bispec_base_size(xsize, ysize, bdepth):
        raise InvalidArgument("bispectrum size does not match (xsize, ysize, bdepth)")
    n = xsize * ysize
    ph = np.zeros(n, np.complex128)
    fl = np.zeros(n, np.uint8)
    cs = np.zeros(n, np.float64)
    _check(_L().smip_reconstruct_phases(device, b.ctypes.data_as(C.POINTER(C.c_float)), xsize, ysize, bdepth,
                                        float(reco_radius), ph.ctypes.data_as(C.POINTER(C.c_double)),
                                        _p(fl, C.c_ubyte), _p(cs, C.c_double)))
    return ph.reshape(ysize, xsize), fl.reshape(ysize, xsize), cs.reshape(ysize, xsize)


def next_reco_index(r: float, phi: float, i: int, j: int):
    """NextRecoIndex (phasereco.cpp:17-36): returns the updated (r, phi, i, j)."""
    r_, p_, i_, j_ = C.c_double(r), C.c_double(phi), C.c_int(i), C.c_int(j)
    _check(_L().smip_next_reco_index(C.byref(r_), C.byref(p_), C.byref(i_), C.byref(j_)))
    return r_.value, p_.value, i_.value, j_.value


def reco_visits(reco_radius: float):
    n = C.c_long()
    _check(_L().smip_reco_visits(float(reco_radius), None, 0, C.byref(n)))
    out = np.zeros((n.value, 2), np.int32)
    _check(_L().smip_reco_visits(float(reco_radius), _p(out, C.c_int), n.value, C.byref(n)))
    return out


def xcorr_displacement_noalloc(ref_ptr: int, frame_ptr: int, ncols: int, nrows: int, shift_ptr: int,
                               stream: int = 0):
    """Shift of the frame against ref, computed without allocating device
    memory (for callers that must not allocate while running).  All three
    pointers are device addresses: ref and frame hold ncols x nrows doubles,
    shift receives two int32 (x, y) on ``stream``.  Frames up to 256 x 256."""
    _check(_L().smip_xcorr_displacement_noalloc(C.c_void_p(ref_ptr), C.c_void_p(frame_ptr), ncols, nrows,
                                                C.c_void_p(shift_ptr), C.c_void_p(stream) if stream else None))


def bispec_offsets(ncols: int, nrows: int, bdepth: int, idx, device: int = 0):
    """Device get_element index path for (n, 4) tuples -> (offsets int64, conj int32)."""
    idx = np.ascontiguousarray(idx, np.int32)
    off = np.zeros(len(idx), np.int64)
    cj = np.zeros(len(idx), np.int32)
    _check(_L().smip_bispec_offsets(device, ncols, nrows, bdepth, _p(idx, C.c_int), len(idx),
                                    off.ctypes.data_as(C.POINTER(C.c_longlong)), _p(cj, C.c_int)))
    return off, cj


def hann(xsize: int, ysize: int, aperture: float, device: int = 0):
    """Hann<double>(xsize, ysize, aperture) as an Array2 in FFT order (ysize, xsize)."""
    out = np.zeros((ysize, xsize), np.float64)
    _check(_L().smip_hann(device, _p(out, C.c_double), xsize, ysize, float(aperture)))
    return out


def shifted(a, dx: int, dy: int, device: int = 0):
    """Array2<double>::shifted({dx, dy}) (array2.h:603-622) on the GPU: the
    (nrows, ncols) array moved by (dx, dy), zero-filled; OutOfRange for a
    distance not smaller than the array."""
    a = np.ascontiguousarray(a, np.float64)
    out = np.zeros_like(a)
    _check(_L().smip_shifted(device, _p(a, C.c_double), _p(out, C.c_double), a.shape[1], a.shape[0], int(dx), int(dy)))
    return out


class CrossCorrelation:
    """CrossCorrelation<double> (include/crosscorrel.h:43-74) on the GPU."""

    def __init__(self, ref, device: int = 0):
        self._ref = np.ascontiguousarray(ref, np.float64)
        self._device = device
        self._corr = None
        self._shift = None

    def correlate(self, frame):
        frame = np.ascontiguousarray(frame, np.float64)
        if frame.shape != self._ref.shape:
            raise InvalidArgument("Matrix dimensions must match for correlation")
        nrows, ncols = frame.shape
        corr = np.zeros_like(frame)
        dx, dy = C.c_int(), C.c_int()
        _check(_L().smip_xcorr_displacement(self._device, _p(self._ref, C.c_double), _p(frame, C.c_double), ncols,
                                            nrows, C.byref(dx), C.byref(dy), _p(corr, C.c_double)))
        self._corr = corr
        self._shift = (dx.value, dy.value)

    def get_correlation_array(self):
        if self._corr is None:
            raise BadFunctionCall("correlation not computed")
        return self._corr

    def get_displacement(self, *args):
        if args:  # static form get_displacement(a, b)
            a, b = args
            return CrossCorrelation(a, self._device if isinstance(self, CrossCorrelation) else 0)(b)
        if self._shift is None:
            raise BadFunctionCall("correlation not computed")
        return self._shift

    def __call__(self, frame):
        self.correlate(frame)
        return self._shift
