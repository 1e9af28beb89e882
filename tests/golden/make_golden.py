"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

Run in a checkout where the reference sources are available:

    make -C oracle ref            # compiles the reference in place into oracle/_ref/
    python tests/golden/make_golden.py

Every expected value below comes from hangeza/speckle-stacker's headers and
sources compiled unmodified (oracle/_ref/libsmip_ref_strict.so = no fast-math,
libsmip_ref_fast.so = the reference's Release flags).  The inputs are seeded
synthetic frames, so the fixtures are reproducible.  The fixtures are read by
tests that run without the reference (CPU oracle tests, GPU parity tests).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "speckle-stacker_gb300"))

from oracle import Reference, bispec_desc  # noqa: E402
from smip_gb300 import synthetic as S  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def stack_fixture(ref_s, ref_f, name, spec, keep_bispec):
    frames = S.make_stack(spec)
    out = ref_s.run_stack(frames, spec.bdepth, spec.reco_radius)
    fast = ref_f.run_stack(frames, spec.bdepth, spec.reco_radius)
    d = bispec_desc(spec.n, spec.n, spec.bdepth)
    rng = np.random.default_rng(7)
    sample = np.sort(rng.choice(d["base_size"], size=min(4096, d["base_size"]), replace=False))
    fx = {
        "frames": frames,
        "bdepth": np.int64(spec.bdepth),
        "reco_radius": np.float64(spec.reco_radius),
        "shifts": out["shifts"],
        "shifts_fast": fast["shifts"],
        "sum": out["sum"],
        "power": out["power"].real.copy(),
        "phases": out["phases"],
        "flags": out["flags"],
        "consistency": out["consistency"],
        "image": out["image"],
        "image_fast": fast["image"],
        "phases_fast": fast["phases"],
        "bispec_sha": np.array(sha(out["bispec"])),
        "bispec_sample_idx": sample.astype(np.int64),
        "bispec_sample": out["bispec"][sample],
    }
    if keep_bispec:
        fx["bispec"] = out["bispec"]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **fx)
    print(name, "frames", frames.shape, frames.dtype, "flags", int(out["flags"].sum()))


def index_fixture(ref_s):
    fx = {}
    for (n, dd) in [(16, 4), (24, 6), (32, 8)]:
        idx = []
        for uy in range(-n // 2, n // 2):
            for ux in range(-n // 2, n // 2):
                for vy in range(-dd // 2, dd // 2 + 1):
                    for vx in range(-dd // 2, dd // 2 + 1):
                        idx.append((ux, uy, vx, vy))
        idx = np.array(idx, np.int32)
        off, cj = ref_s.get_element_offsets(n, n, dd, idx)
        fx[f"n{n}_d{dd}_idx"] = idx
        fx[f"n{n}_d{dd}_off"] = off.astype(np.int64)
        fx[f"n{n}_d{dd}_conj"] = cj.astype(np.int8)
    # descriptor cases incl. the reference unit test (bispectrum_test.cpp:33-41)
    desc = []
    for (nc, nr, dd) in [(2, 3, 4), (3, 4, 5), (4, 4, 4), (32, 32, 8), (64, 64, 16), (128, 128, 32),
                         (256, 256, 32), (512, 512, 48), (255, 129, 31)]:
        r = ref_s.describe(nc, nr, dd)
        desc.append([nc, nr, dd] + list(r["sizes"]) + list(r["base_sizes"]) + [r["base_size"], r["totalsize"]]
                    + list(r["min"]) + list(r["max"]))
    fx["describe"] = np.array(desc, np.int64)
    np.savez_compressed(os.path.join(HERE, "bispec_index.npz"), **fx)
    print("bispec_index", {k: v.shape for k, v in fx.items()})


def visits_fixture(ref_s, ref_f):
    fx = {}
    for R in (12, 24, 32, 64, 128, 200):
        v = ref_s.reco_visits(R)
        vf = ref_f.reco_visits(R)
        assert np.array_equal(v, vf)
        fx[f"r{R}_count"] = np.int64(len(v))
        fx[f"r{R}_sha"] = np.array(sha(v.astype(np.int32)))
        if R <= 64:
            fx[f"r{R}"] = v.astype(np.int16)
    np.savez_compressed(os.path.join(HERE, "reco_visits.npz"), **fx)
    print("reco_visits", {k: (v.shape if hasattr(v, "shape") else v) for k, v in fx.items() if not k.endswith("sha")})


def xcorr_fixture(ref_s, ref_f):
    """tests/correl_test.cpp restated with a fixed seed: a 128^2 Gaussian
    (sigma 5) shifted by random integer shifts; the reference's measured shifts."""
    n, sigma = 128, 5.0
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    # smip::Gauss with params {sigma*2*3.14, sigma}, {n/2, n/2}, {sigma, sigma}
    # (math_functions.h:46-59): prod over axes of p0*exp(-(x-p1)^2/(2 p2^2))/(p2*sqrt(2 pi))
    c2pi = 2.5070831590532e00
    p0 = sigma * 2.0 * 3.14
    gx = p0 * np.exp(-((xx - n / 2) ** 2) / (sigma * sigma * 2)) / (sigma * c2pi)
    gy = p0 * np.exp(-((yy - n / 2) ** 2) / (sigma * sigma * 2)) / (sigma * c2pi)
    gaus = gx * gy
    rng = np.random.default_rng(12345)
    lo, hi = -(n // 2) + int(sigma), (n // 2 - 1) - int(sigma) - 1
    gen = rng.integers(lo, hi + 1, size=(32, 2))
    frames = np.stack([ref_s.shifted(gaus, int(dx), int(dy)) for dx, dy in gen])
    meas = np.array([ref_s.xcorr(gaus, f) for f in frames], np.int32)
    meas_f = np.array([ref_f.xcorr(gaus, f) for f in frames], np.int32)
    # frames are exact zero-filled shifts of gaus (Array2::shifted), so only
    # gaus and the shifts are stored
    np.savez_compressed(os.path.join(HERE, "xcorr_gauss.npz"), gaus=gaus,
                        generated=gen.astype(np.int32), measured=meas, measured_fast=meas_f)
    print("xcorr_gauss exact", int((meas == gen).all(axis=1).sum()), "/", len(gen))


def main():
    if not (Reference.available("strict") and Reference.available("fast")):
        raise SystemExit("build the reference first: make -C oracle ref")
    ref_s, ref_f = Reference("strict"), Reference("fast")
    stack_fixture(ref_s, ref_f, "stack_binary32_u8",
                  S.StackSpec(n=32, nframes=8, kind="binary", dtype="uint8", d_over_r0=4.0,
                              bdepth=8, reco_radius=12, seed=31), keep_bispec=True)
    stack_fixture(ref_s, ref_f, "stack_ext64_u16",
                  S.StackSpec(n=64, nframes=6, kind="extended", dtype="uint16", d_over_r0=6.0,
                              bdepth=16, reco_radius=24, seed=61, nblobs=8), keep_bispec=False)
    index_fixture(ref_s)
    visits_fixture(ref_s, ref_f)
    xcorr_fixture(ref_s, ref_f)


if __name__ == "__main__":
    main()
