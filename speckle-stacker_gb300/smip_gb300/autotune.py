"""Autotuner of the frame batch and of the bispectrum kernel's staging and
tile split.

A stack accumulates its frames in batches of ``batch_frames``: every batch is
one pass of the FFT kernels and one launch of the bispectrum kernel, whose
packed accumulator (read and written once per launch) and work split (tiles
per SM, frames per split part) depend on the batch size.  The library's
default is about 2 GB of batch buffers (1024 frames at 256x256 and below).
The kernel itself has two tunables (Stack.set_kernel_config): the frames
staged per shared-memory ring stage (four or two: ``variant`` 0 or 1) and the
fewest frames per part when the last partial wave of tiles is split by frames
(``min_part``).  This module times candidate batch sizes for a shape on the
device at hand, then the kernel tunables at the best batch size, keeps the
fastest and caches it per (device, shape, depth, dtype) in a JSON file next to
the package, so ``Stack(..., batch_frames="auto")`` pays for the search once.
"""
from __future__ import annotations

import json
import os
import threading
import time

import numpy as np

CACHE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), ".autotune.json")
CANDIDATES = (32, 64, 128, 256, 512, 1024)
KERNEL_CANDIDATES = ((0, 0), (1, 0), (0, 32), (1, 32), (0, 1 << 30))  # (variant, min_part); 1 << 30: no split
_lock = threading.Lock()


def _key(device_name: str, ncols: int, nrows: int, bdepth: int, dtype: str) -> str:
    return f"{device_name}|{ncols}x{nrows}|d{(bdepth // 2) * 2}|{dtype}"


def _device_name(device: int) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:  # pragma: no cover - torch without CUDA
        return f"cuda{device}"


def _load() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table: dict):
    tmp = CACHE + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def spectra_bytes_per_frame(ncols: int, nrows: int) -> int:
    """Device bytes one batched frame holds (row spectra in float-float,
    spectra, correlation columns and rows), which bounds the batch size."""
    hw = ncols // 2 + 1
    return hw * nrows * (16 + 8 + 8) + ncols * nrows * 4


def measure(ncols: int, nrows: int, bdepth: int, batch_frames: int, frames: np.ndarray, device: int = 0,
            repeats: int = 2, kernel=(0, 0)) -> float:
    """frames/s of pushing ``frames`` (already batched in ``batch_frames``)
    with the kernel tunables ``kernel`` = (variant, min_part)."""
    from smip_gb300 import Stack

    with Stack(ncols, nrows, bdepth, device=device, batch_frames=batch_frames) as st:
        st.set_kernel_config(*kernel)
        st.push_frames(frames)  # warm-up (allocations, first launch)
        st.sync()
        best = 0.0
        for _ in range(repeats):
            st.reset()
            t0 = time.perf_counter()
            st.push_frames(frames)
            st.flush()
            st.sync()
            best = max(best, len(frames) / (time.perf_counter() - t0))
    return best


def tune(ncols: int, nrows: int, bdepth: int, dtype=np.uint16, device: int = 0, candidates=None,
         mem_limit: float = 8e9, seed: int = 99) -> dict:
    """Times every candidate batch size (those whose batch buffers fit in
    ``mem_limit`` bytes) on 2 x the largest candidate's frames of seeded noise;
    returns {"batch_frames": best, "frames_per_s": {candidate: rate}}."""
    candidates = CANDIDATES if candidates is None else candidates
    per = spectra_bytes_per_frame(ncols, nrows)
    cands = [c for c in candidates if c * per <= mem_limit] or [min(candidates)]
    n = 2 * max(cands)
    rng = np.random.default_rng(seed)
    hi = 255 if np.dtype(dtype) == np.uint8 else 4095
    frames = rng.integers(0, hi, (n, nrows, ncols)).astype(dtype)
    rates = {c: measure(ncols, nrows, bdepth, c, frames, device) for c in cands}
    best = max(rates, key=rates.get)
    krates = {k: measure(ncols, nrows, bdepth, best, frames, device, kernel=k) for k in KERNEL_CANDIDATES}
    kbest = max(krates, key=krates.get)
    return {"batch_frames": int(best), "frames_per_s": {str(k): v for k, v in rates.items()},
            "variant": int(kbest[0]), "min_part": int(kbest[1]),
            "kernel_frames_per_s": {f"{k[0]}/{k[1]}": v for k, v in krates.items()}}


def best_config(ncols: int, nrows: int, bdepth: int, dtype=np.uint16, device: int = 0) -> dict:
    """The cached best {batch_frames, variant, min_part} for this device and
    shape, tuning on first use."""
    key = _key(_device_name(device), ncols, nrows, bdepth, np.dtype(dtype).name)
    with _lock:
        table = _load()
        if key not in table or "variant" not in table[key]:
            table = _load()
            table[key] = tune(ncols, nrows, bdepth, dtype, device)
            _store(table)
        e = table[key]
        return {"batch_frames": int(e["batch_frames"]), "variant": int(e.get("variant", 0)),
                "min_part": int(e.get("min_part", 0))}


def best_batch(ncols: int, nrows: int, bdepth: int, dtype=np.uint16, device: int = 0) -> int:
    """The cached best batch size for this device and shape, tuning on first use."""
    return best_config(ncols, nrows, bdepth, dtype, device)["batch_frames"]


def main(argv=None):
    """Times one configuration: python -m smip_gb300.autotune NCOLS NROWS DEPTH
    [--frames N] [--batch B] [--variant V] [--min-part P] [--repeats R];
    prints frames/s of the whole per-frame pipeline and of the bispectrum
    kernel alone (CUDA events) on seeded noise frames."""
    import argparse

    ap = argparse.ArgumentParser(prog="python -m smip_gb300.autotune")
    ap.add_argument("ncols", type=int)
    ap.add_argument("nrows", type=int)
    ap.add_argument("depth", type=int)
    ap.add_argument("--frames", type=int, default=1024)
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--min-part", type=int, default=0)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    from smip_gb300 import Stack

    rng = np.random.default_rng(99)
    frames = rng.integers(0, 4095, (a.frames, a.nrows, a.ncols)).astype(np.uint16)
    with Stack(a.ncols, a.nrows, a.depth, device=a.device, batch_frames=a.batch) as st:
        st.set_kernel_config(a.variant, a.min_part)
        st.push_frames(frames)  # warm-up
        st.sync()
        st.kernel_time()
        st.set_timing(True)
        t0 = time.perf_counter()
        for _ in range(a.repeats):
            st.reset()
            st.push_frames(frames)
            st.flush()
        st.sync()
        el = time.perf_counter() - t0
        ms, n, fr = st.kernel_time()
    print(json.dumps({"shape": [a.ncols, a.nrows, a.depth], "variant": a.variant, "min_part": a.min_part,
                      "pipeline_frames_per_s": a.frames * a.repeats / el,
                      "bispec_kernel_frames_per_s": fr / (ms * 1e-3) if ms > 0 else None,
                      "bispec_launches": n}))


if __name__ == "__main__":
    main()
