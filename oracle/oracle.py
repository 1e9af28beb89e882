"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries sit behind the same Python surface:

* ``Oracle()`` -- the plain-C restatement in ``oracle/smip_oracle.c``
  (built into ``oracle/_build/``).  It is available everywhere, including
  machines without the reference sources.
* ``Reference(flavour)`` -- the reference's own headers compiled in place by
  ``make -C oracle ref`` into ``oracle/_ref/`` (``strict`` = no fast-math,
  ``fast`` = the reference's Release flags).  Only present where the
  reference sources were available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this
module; the CUDA library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference source tree (read only by the build recipe and by tests that
# use its sample data); the SMIP_REFERENCE environment variable overrides it.
REFERENCE = os.environ.get("SMIP_REFERENCE", "/root/reference")
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")

DTYPES = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.float32): 2, np.dtype(np.float64): 3}

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)
_ubp = C.POINTER(C.c_ubyte)


def build(reference: str | None = None) -> None:
    """Compile the oracle (and the reference build when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref = reference or REFERENCE
    if os.path.isdir(os.path.join(ref, "include")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={ref}"], check=True)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def bispec_desc(ncols, nrows, depth):
    """Packed-bispectrum descriptor (include/bispectrum.h:143-160, 203-220)."""
    sizes = [(d // 2) * 2 + 1 for d in (ncols, nrows, depth, depth)]
    base = [s - s // 2 if n in (0, 2) else s for n, s in enumerate(sizes)]
    mins = [-(s // 2) for s in sizes]
    maxs = [s + m - 1 for s, m in zip(sizes, mins)]
    bs = base[0] * base[1] * base[2] * base[3]
    return {"sizes": sizes, "base_sizes": base, "base_size": bs,
            "totalsize": sizes[0] * sizes[1] * sizes[2] * sizes[3], "min": mins, "max": maxs}


class _Common:
    """Wrappers shared by the oracle and the reference build."""

    lib: C.CDLL
    prefix: str

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    # ---- FFT-order helpers -------------------------------------------------
    @staticmethod
    def as_c128(a):
        return np.ascontiguousarray(a, dtype=np.complex128)

    def accumulate(self, B, fft, depth, fp64=False, nthreads=1):
        """B += triple products of one spectrum (bispectrum.h:356-409), in place."""
        nrows, ncols = fft.shape
        fft = self.as_c128(fft)
        if fp64:
            assert B.dtype == np.complex128
            self._acc64(B, fft, ncols, nrows, depth, nthreads)
        else:
            assert B.dtype == np.complex64
            self._acc32(B, fft, ncols, nrows, depth, nthreads)
        return B

    def reconstruct_phases(self, B, xsize, ysize, depth, reco_radius):
        np_ = xsize * ysize
        ph = np.zeros(np_, np.complex128)
        fl = np.zeros(np_, np.uint8)
        cs = np.zeros(np_, np.float64)
        rc = self._reco(B, xsize, ysize, depth, float(reco_radius), ph, fl, cs)
        if rc != 0:
            raise IndexError("reconstruct_phases: bispectrum element out of range")
        return ph.reshape(ysize, xsize), fl.reshape(ysize, xsize), cs.reshape(ysize, xsize)

    def xcorr(self, ref, frame, want_corr=False):
        nrows, ncols = ref.shape
        ref = np.ascontiguousarray(ref, np.float64)
        frame = np.ascontiguousarray(frame, np.float64)
        dx, dy = C.c_int(), C.c_int()
        corr = np.zeros((nrows, ncols), np.float64) if want_corr else None
        self._xcorr(ref, frame, ncols, nrows, dx, dy, corr)
        return ((dx.value, dy.value), corr) if want_corr else (dx.value, dy.value)

    def shifted(self, a, dx, dy):
        nrows, ncols = a.shape
        a = np.ascontiguousarray(a, np.float64)
        out = np.zeros_like(a)
        self._f("shifted")(_ptr(a, _dp), _ptr(out, _dp), ncols, nrows, dx, dy)
        return out

    def next_reco_index(self, r, phi, i, j):
        r_, p_, i_, j_ = C.c_double(r), C.c_double(phi), C.c_int(i), C.c_int(j)
        self._f("next_reco_index")(C.byref(r_), C.byref(p_), C.byref(i_), C.byref(j_))
        return r_.value, p_.value, i_.value, j_.value

    def run_stack(self, frames, depth, reco_radius, fp64=False, nthreads=1):
        """Whole pipeline (smip-cli/main.cpp:246-378).  frames: (n, nrows, ncols)."""
        frames = np.ascontiguousarray(frames)
        n, nrows, ncols = frames.shape
        npx = nrows * ncols
        d = bispec_desc(ncols, nrows, depth)
        out = {
            "shifts": np.zeros((n, 2), np.int32),
            "sum": np.zeros((nrows, ncols), np.float64),
            "power": np.zeros((nrows, ncols), np.complex128),
            "phases": np.zeros((nrows, ncols), np.complex128),
            "flags": np.zeros((nrows, ncols), np.uint8),
            "consistency": np.zeros((nrows, ncols), np.float64),
            "image": np.zeros((nrows, ncols), np.complex128),
        }
        b32 = None if fp64 else np.zeros(d["base_size"], np.complex64)
        b64 = np.zeros(d["base_size"], np.complex128) if fp64 else None
        rc = self._run(frames, DTYPES[frames.dtype], n, ncols, nrows, depth, float(reco_radius), int(fp64),
                       nthreads, out, b32, b64)
        if rc != 0:
            raise RuntimeError(f"run_stack failed: {rc}")
        out["bispec"] = b64 if fp64 else b32
        _ = npx
        return out


class Oracle(_Common):
    prefix = "orc_"

    def __init__(self, path: str | None = None):
        path = path or os.path.join(BUILD_DIR, "libsmip_oracle.so")
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_calc_offset.restype = C.c_long
        L.orc_get_element_offset.restype = C.c_long
        L.orc_reco_visits.restype = C.c_long
        for n in ("orc_accumulate_f32", "orc_accumulate_f64"):
            getattr(L, n).argtypes = [C.c_void_p, _dp, C.c_long, C.c_long, C.c_long, C.c_int]
        L.orc_reconstruct_phases.argtypes = [_fp, _dp, C.c_long, C.c_long, C.c_long, C.c_double, _dp, _ubp, _dp]
        L.orc_xcorr_displacement.argtypes = [_dp, _dp, C.c_long, C.c_long, _ip, _ip, _dp]
        L.orc_shifted.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_int, C.c_int]
        L.orc_general_hamming.argtypes = [_dp, C.c_long, C.c_long, C.c_double, C.c_double]
        L.orc_fft_2d.argtypes = [_dp, C.c_long, C.c_long, C.c_int]
        L.orc_map_to_color_u16.argtypes = [_dp, C.c_long, C.POINTER(C.c_uint16)]
        L.orc_array2mat_order.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_int]
        L.orc_fft_r2c_2d.argtypes = [_dp, _dp, C.c_long, C.c_long]
        L.orc_fft_c2r_2d.argtypes = [_dp, _dp, C.c_long, C.c_long]
        L.orc_run_stack.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_long, C.c_long, C.c_double,
                                    C.c_int, C.c_int, _ip, _dp, _dp, _fp, _dp, _dp, _ubp, _dp, _dp]
        L.orc_accumulate_frames.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_long, C.c_long,
                                            C.c_int, _dp, _fp, _dp, _dp, _ip]

    def _acc32(self, B, fft, ncols, nrows, depth, nthreads):
        self.lib.orc_accumulate_f32(B.ctypes.data, _ptr(fft, _dp), ncols, nrows, depth, nthreads)

    def _acc64(self, B, fft, ncols, nrows, depth, nthreads):
        self.lib.orc_accumulate_f64(B.ctypes.data, _ptr(fft, _dp), ncols, nrows, depth, nthreads)

    def _reco(self, B, xs, ys, depth, R, ph, fl, cs):
        if B.dtype == np.complex64:
            return self.lib.orc_reconstruct_phases(_ptr(B, _fp), None, xs, ys, depth, R,
                                                   _ptr(ph, _dp), _ptr(fl, _ubp), _ptr(cs, _dp))
        return self.lib.orc_reconstruct_phases(None, _ptr(B, _dp), xs, ys, depth, R,
                                               _ptr(ph, _dp), _ptr(fl, _ubp), _ptr(cs, _dp))

    def _xcorr(self, ref, frame, ncols, nrows, dx, dy, corr):
        self.lib.orc_xcorr_displacement(_ptr(ref, _dp), _ptr(frame, _dp), ncols, nrows,
                                        C.byref(dx), C.byref(dy), _ptr(corr, _dp))

    def _run(self, frames, dt, n, ncols, nrows, depth, R, fp64, nthreads, out, b32, b64):
        return self.lib.orc_run_stack(frames.ctypes.data, dt, n, ncols, nrows, depth, R, fp64, nthreads,
                                      _ptr(out["shifts"], _ip), _ptr(out["sum"], _dp), _ptr(out["power"], _dp),
                                      _ptr(b32, _fp), _ptr(b64, _dp), _ptr(out["phases"], _dp),
                                      _ptr(out["flags"], _ubp), _ptr(out["consistency"], _dp),
                                      _ptr(out["image"], _dp))

    # ---- oracle-only helpers ----------------------------------------------
    def get_element_offsets(self, ncols, nrows, depth, idx):
        """idx: (n,4) int array -> (offsets, conj); offset -1 where the reference throws."""
        idx = np.ascontiguousarray(idx, np.int32)
        d = (C.c_long * 24)()
        self.lib.orc_bispec_describe(C.c_long(ncols), C.c_long(nrows), C.c_long(depth), C.c_long(depth), d)
        off = np.empty(len(idx), np.int64)
        cj = np.empty(len(idx), np.int32)
        c = C.c_int()
        for q in range(len(idx)):
            off[q] = self.lib.orc_get_element_offset(d, idx[q].ctypes.data_as(_ip), C.byref(c))
            cj[q] = c.value
        return off, cj

    def reco_visits(self, reco_radius):
        n = self.lib.orc_reco_visits(C.c_double(reco_radius), None, C.c_long(0))
        out = np.zeros((n, 2), np.int32)
        self.lib.orc_reco_visits(C.c_double(reco_radius), _ptr(out, _ip), C.c_long(n))
        return out

    def hann(self, xsize, ysize, aperture, alpha=0.5):
        out = np.zeros((ysize, xsize), np.float64)
        self.lib.orc_general_hamming(_ptr(out, _dp), xsize, ysize, float(aperture), float(alpha))
        return out

    def map_to_color(self, v):
        """mapToColor<uint16_t> (videoio.h:178-206) of every value: (..., 3) r, g, b."""
        v = np.ascontiguousarray(v, np.float64)
        out = np.zeros(v.shape + (3,), np.uint16)
        self.lib.orc_map_to_color_u16(_ptr(v, _dp), v.size, out.ctypes.data_as(C.POINTER(C.c_uint16)))
        return out

    def array2mat_order(self, a, signed_symmetry):
        """Array2Mat's pixel order (videoio.h:137-146) of a real (nrows, ncols) array."""
        a = np.ascontiguousarray(a, np.float64)
        out = np.zeros_like(a)
        self.lib.orc_array2mat_order(_ptr(a, _dp), _ptr(out, _dp), a.shape[1], a.shape[0], int(signed_symmetry))
        return out

    def fft2(self, a, sign=-1):
        a = np.array(a, dtype=np.complex128, copy=True, order="C")
        self.lib.orc_fft_2d(_ptr(a, _dp), a.shape[0], a.shape[1], sign)
        return a

    def accumulate_frames(self, frames, depth, ref_frame, B, power, sumacc, nthreads=1):
        """Per-frame pipeline on frames (n, nrows, ncols) continuing the given accumulators."""
        frames = np.ascontiguousarray(frames)
        n, nrows, ncols = frames.shape
        shifts = np.zeros((n, 2), np.int32)
        self.lib.orc_accumulate_frames(frames.ctypes.data, DTYPES[frames.dtype], n, ncols, nrows, depth, nthreads,
                                       _ptr(np.ascontiguousarray(ref_frame, np.float64), _dp), _ptr(B, _fp),
                                       _ptr(power, _dp), _ptr(sumacc, _dp), _ptr(shifts, _ip))
        return shifts


class Reference(_Common):
    """The reference's own code, compiled in place (oracle/_ref)."""

    prefix = "ref_"

    @staticmethod
    def available(flavour: str = "strict") -> bool:
        return os.path.exists(os.path.join(REF_DIR, f"libsmip_ref_{flavour}.so"))

    def __init__(self, flavour: str = "strict"):
        self.lib = C.CDLL(os.path.join(REF_DIR, f"libsmip_ref_{flavour}.so"))
        L = self.lib
        L.ref_calc_offset.restype = C.c_long
        L.ref_bispec_read.restype = C.c_long
        L.ref_accumulate_f32.argtypes = [_fp, _dp, C.c_long, C.c_long, C.c_long]
        L.ref_accumulate_f64.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_long]
        L.ref_reconstruct_phases_f32.argtypes = [_fp, C.c_long, C.c_long, C.c_long, C.c_double, _dp, _ubp, _dp]
        L.ref_reconstruct_phases_f64.argtypes = [_dp, C.c_long, C.c_long, C.c_long, C.c_double, _dp, _ubp, _dp]
        L.ref_xcorr.argtypes = [_dp, _dp, C.c_long, C.c_long, _ip, _ip, _dp]
        L.ref_shifted.argtypes = [_dp, _dp, C.c_long, C.c_long, C.c_int, C.c_int]
        L.ref_hann.argtypes = [_dp, C.c_long, C.c_long, C.c_double]
        L.ref_get_element_probe.argtypes = [C.c_long, C.c_long, C.c_long, _ip, C.c_long, _lp, _ip]
        L.ref_describe.argtypes = [C.c_long, C.c_long, C.c_long, _lp]
        L.ref_run_stack.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_long, C.c_long, C.c_double,
                                    C.c_int, _ip, _dp, _dp, _fp, _dp, _dp, _ubp, _dp, _dp]
        L.ref_bispec_write.argtypes = [C.c_char_p, _fp, C.c_long, C.c_long, C.c_long]
        L.ref_bispec_read.argtypes = [C.c_char_p, _fp, C.c_long, _lp]
        L.ref_calc_indices.argtypes = [C.c_long, C.c_long, C.c_long, C.c_long, _ip]
        L.ref_calc_offset.argtypes = [C.c_long, C.c_long, C.c_long, _ip]

    def _acc32(self, B, fft, ncols, nrows, depth, nthreads):
        self.lib.ref_accumulate_f32(_ptr(B, _fp), _ptr(fft, _dp), ncols, nrows, depth)

    def _acc64(self, B, fft, ncols, nrows, depth, nthreads):
        self.lib.ref_accumulate_f64(_ptr(B, _dp), _ptr(fft, _dp), ncols, nrows, depth)

    def _reco(self, B, xs, ys, depth, R, ph, fl, cs):
        if B.dtype == np.complex64:
            return self.lib.ref_reconstruct_phases_f32(_ptr(B, _fp), xs, ys, depth, R,
                                                       _ptr(ph, _dp), _ptr(fl, _ubp), _ptr(cs, _dp))
        return self.lib.ref_reconstruct_phases_f64(_ptr(B, _dp), xs, ys, depth, R,
                                                   _ptr(ph, _dp), _ptr(fl, _ubp), _ptr(cs, _dp))

    def _xcorr(self, ref, frame, ncols, nrows, dx, dy, corr):
        self.lib.ref_xcorr(_ptr(ref, _dp), _ptr(frame, _dp), ncols, nrows, C.byref(dx), C.byref(dy),
                           _ptr(corr, _dp))

    def _run(self, frames, dt, n, ncols, nrows, depth, R, fp64, nthreads, out, b32, b64):
        return self.lib.ref_run_stack(frames.ctypes.data, dt, n, ncols, nrows, depth, R, fp64,
                                      _ptr(out["shifts"], _ip), _ptr(out["sum"], _dp), _ptr(out["power"], _dp),
                                      _ptr(b32, _fp), _ptr(b64, _dp), _ptr(out["phases"], _dp),
                                      _ptr(out["flags"], _ubp), _ptr(out["consistency"], _dp),
                                      _ptr(out["image"], _dp))

    def describe(self, ncols, nrows, depth):
        out = np.zeros(18, np.int64)
        self.lib.ref_describe(ncols, nrows, depth, out.ctypes.data_as(_lp))
        return {"sizes": list(out[0:4]), "base_sizes": list(out[4:8]), "base_size": int(out[8]),
                "totalsize": int(out[9]), "min": list(out[10:14]), "max": list(out[14:18])}

    def get_element_offsets(self, ncols, nrows, depth, idx):
        idx = np.ascontiguousarray(idx, np.int32)
        off = np.empty(len(idx), np.int64)
        cj = np.empty(len(idx), np.int32)
        self.lib.ref_get_element_probe(ncols, nrows, depth, _ptr(idx, _ip), len(idx),
                                       off.ctypes.data_as(_lp), _ptr(cj, _ip))
        return off, cj

    def hann(self, xsize, ysize, aperture):
        out = np.zeros((ysize, xsize), np.float64)
        if self.lib.ref_hann(_ptr(out, _dp), xsize, ysize, float(aperture)) != 0:
            raise ValueError("WindowFunction aperture size <= 0")
        return out

    def reco_visits(self, reco_radius):
        out = []
        r, phi, i, j = 0.0, 0.0, 0, 0
        while r <= reco_radius:
            r, phi, i, j = self.next_reco_index(r, phi, i, j)
            out.append((i, j))
        return np.array(out, np.int32)

    def write_bispec(self, fn, B, ncols, nrows, depth):
        return self.lib.ref_bispec_write(fn.encode(), _ptr(np.ascontiguousarray(B, np.complex64), _fp),
                                         ncols, nrows, depth)

    def read_bispec(self, fn, cap):
        B = np.zeros(cap, np.complex64)
        dims = np.zeros(4, np.int64)
        n = self.lib.ref_bispec_read(fn.encode(), _ptr(B, _fp), cap, dims.ctypes.data_as(_lp))
        return n, B, dims
