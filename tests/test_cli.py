"""smip-cli (speckle-stacker_gb300/cli/smip_cli.cpp) and the C++ layer
(speckle-stacker_gb300/include/smip/gpu.hpp): the reference's command line and
C++ call pattern over the C ABI.

CPU tests check the command line without a device and that a C++ program
builds against the header layer; GPU tests run both and compare every output
with the ctypes binding, which the parity tests check against the oracle."""
import os
import shutil
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "speckle-stacker_gb300")
CLI = os.path.join(PKG, "bin", "smip-cli")


def _need_cli():
    if not os.path.exists(CLI):
        pytest.skip("smip-cli not built (make -C speckle-stacker_gb300)")


def read_png16(path):
    """Minimal reader for the CLI's 16-bit gray/RGB PNGs (stored or deflated)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(typ + body)
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype = ihdr[:4]
    assert depth == 16 and ctype in (0, 2)
    ch = 3 if ctype == 2 else 1
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + w * ch * 2)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].copy().view(">u2").astype(np.uint16).reshape(h, w, ch)[..., 0 if ch == 1 else slice(None)]


def test_cli_version_and_help():
    _need_cli()
    out = subprocess.run([CLI, "--version"], capture_output=True, text=True, check=True)
    assert "v0.3.2" in out.stdout
    out = subprocess.run([CLI, "-h"], capture_output=True, text=True, check=True)
    for flag in ("--nrframes", "--refframe", "--recoradius", "--bdepth", "--channel", "--croppos", "--cropsize",
                 "--no-calcsum", "--no-specklemasking", "--verbose", "--version"):
        assert flag in out.stdout
    # no source: usage, exit 0 (main.cpp:215-218)
    assert subprocess.run([CLI], capture_output=True).returncode == 0


def test_cli_rejects_bad_input(tmp_path):
    _need_cli()
    bad = tmp_path / "x.npy"
    np.save(bad, np.zeros((2, 16, 16), np.int32))
    r = subprocess.run([CLI, str(bad)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "unsupported dtype" in r.stderr
    r = subprocess.run([CLI, str(tmp_path / "missing.npy")], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "file open error" in r.stderr
    r = subprocess.run([CLI, "-k", "-1:3", str(bad)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "crop box" in r.stderr


def test_cli_apply_ignored_checks_arguments(tmp_path):
    """--apply-ignored makes -r, -k and -s take effect; a crop box outside the
    frame or a reference frame past the last one is an error before any device
    work (without the switch both are ignored, as in the reference)."""
    _need_cli()
    out = subprocess.run([CLI, "-h"], capture_output=True, text=True, check=True)
    assert "--apply-ignored" in out.stdout and "--rings" in out.stdout
    src = tmp_path / "s.npy"
    np.save(src, np.zeros((2, 32, 32), np.uint8))
    r = subprocess.run([CLI, "--apply-ignored", "-k", "20:0", "-s", "16:16", str(src)], capture_output=True,
                       text=True, cwd=tmp_path)
    assert r.returncode == 1 and "crop box outside the frame" in r.stderr
    r = subprocess.run([CLI, "--apply-ignored", "-r", "2", str(src)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "reference frame index out of range" in r.stderr


def _build_api_check(out_dir):
    exe = os.path.join(out_dir, "api_check")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(PKG, "include"), os.path.join(ROOT, "tests", "cpp", "api_check.cpp"),
           "-L" + os.path.join(PKG, "lib"), "-lsmip_gpu", "-Wl,-rpath," + os.path.join(PKG, "lib"), "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_layer_builds(tmp_path):
    if shutil.which("g++") is None or not os.path.exists(os.path.join(PKG, "lib", "libsmip_gpu.so")):
        pytest.skip("g++ or libsmip_gpu.so missing")
    assert os.path.exists(_build_api_check(str(tmp_path)))


@pytest.mark.gpu
def test_cli_matches_binding(smip, oracle, tmp_path):
    """smip-cli -b 20 -p 40 -n 10 on a 12-frame u8 stack: bispectrum.dat and every
    PNG equal what the binding gives for the same frames (default depth 20)."""
    _need_cli()
    from smip_gb300 import synthetic as S

    frames = S.make_stack(S.config_spec("binary128", nframes=12))
    src = tmp_path / "stack.npy"
    np.save(src, frames)
    r = subprocess.run([CLI, "-b", "20", "-p", "40", "-n", "10", str(src)], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    used = frames[:10]
    n = used.shape[1]
    with smip.Stack(n, n, 20) as st:
        st.push_frames(used)
        ref_dat = tmp_path / "ref.dat"
        st.save_bispectrum(str(ref_dat))
        img, ph, fl, cons = st.finish(40.0)
        sm, pw = st.sum(), st.power()
    assert open(tmp_path / "bispectrum.dat", "rb").read() == open(ref_dat, "rb").read()
    win = smip.hann(n, n, 80.0)

    def gray(v):
        return np.clip(v * 65535.0, 0, 65535).astype(np.uint16)

    def shift(a):  # signed_symmetry: pixel (x, y) shows element (x - n/2, y - n/2)
        return np.roll(a, (n // 2, n // 2), axis=(0, 1))

    exp = {
        "sum_image.png": gray(np.abs(sm / 255.0)),
        "reco_image.png": gray(shift(np.abs(img))),
        "phases.png": gray(shift((np.angle(ph * win) + np.pi) / (2 * np.pi))),
        "powerspec.png": gray(shift(np.abs(pw / (np.abs(pw).max() / 1000.0)))),
    }
    for name, e in exp.items():
        got = read_png16(tmp_path / name)
        assert got.shape == e.shape
        assert np.abs(got.astype(np.int64) - e.astype(np.int64)).max() <= 1, name
    # false colour: the oracle's mapToColor (videoio.h:178-206) in Array2Mat's
    # pixel order (videoio.h:137-146) of the same values
    colour = {
        "sum_image_falsecolor.png": (np.abs(sm / 255.0), False),
        "phases_falsecolor.png": ((np.angle(ph * win) + np.pi) / (2 * np.pi), True),
        "phasecons.png": (cons, True),
        "powerspec_falsecolor.png": (np.abs(pw / (np.abs(pw).max() / 1000.0)), True),
        "reco_image_falsecolor.png": (np.abs(img), True),
    }
    for name, (vals, signed) in colour.items():
        e = oracle.map_to_color(oracle.array2mat_order(vals, signed))
        got = read_png16(tmp_path / name)
        assert got.shape == (n, n, 3), name
        assert np.abs(got.astype(np.int64) - e.astype(np.int64)).max() <= 1, name


@pytest.mark.gpu
def test_cpp_layer_matches_binding(smip, tmp_path):
    """The C++ layer's Stack, Bispectrum, reconstruct_phases, CrossCorrelation,
    Hann and NextRecoIndex against the binding on the same inputs."""
    exe = _build_api_check(str(tmp_path))
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, (r.returncode, r.stdout, r.stderr)
    # the same frames: std::mt19937(5) outputs % 4096, 6 frames of 64x64, row-major
    # (numpy's legacy RandomState is the same MT19937 with the same integer seeding)
    vals = np.random.RandomState(5).randint(0, 2 ** 32, size=6 * 64 * 64, dtype=np.uint32)
    frames = (vals % 4096).astype(np.float64).reshape(6, 64, 64)
    dx, dy = np.fromfile(tmp_path / "xc_shift.bin", np.int32)
    assert (dx, dy) == smip.CrossCorrelation(frames[0])(frames[1])
    with smip.Stack(64, 64, 20) as st:
        st.push_frames(frames)
        b = st.bispectrum()
        ph, fl, _ = st.reconstruct_phases(24.0)
    assert np.array_equal(np.fromfile(tmp_path / "stack_bispec.bin", np.complex64), b)
    assert np.array_equal(np.fromfile(tmp_path / "stack_phases.bin", np.complex128), ph.ravel())
    assert np.array_equal(np.fromfile(tmp_path / "stack_flags.bin", np.uint8), fl.ravel())
    assert tuple(np.fromfile(tmp_path / "next_reco.bin", np.int32)) == smip.next_reco_index(0.0, 0.0, 0, 0)[2:]
    assert np.array_equal(np.fromfile(tmp_path / "hann.bin", np.float64), smip.hann(64, 64, 48.0).ravel())
    assert np.array_equal(np.fromfile(tmp_path / "shifted.bin", np.float64), smip.shifted(frames[0], 3, -2).ravel())


@pytest.mark.gpu
def test_cli_reads_animated_gif(smip, tmp_path):
    """An animated GIF through smip-cli equals the same frames given as .npy:
    frames in BGR as OpenCV delivers them, -c r reading channel 0 (blue) and
    -c b channel 2 (red), as Mat2Array's channel = round(log2(c)) does."""
    _need_cli()
    from smip_gb300 import synthetic as S
    from test_gif import write_gif

    idx = S.make_stack(S.config_spec("binary128", nframes=8, n=64)).astype(np.int64)  # u8 values as palette indices
    pal = np.stack([np.arange(256), 255 - np.arange(256), (np.arange(256) * 7) % 256], axis=1)  # R, G, B
    gif = tmp_path / "stack.gif"
    write_gif(str(gif), 64, 64, [{"idx": f, "disposal": 1} for f in idx], gct=pal)
    for flag, plane in (("r", pal[:, 2]), ("b", pal[:, 0])):
        d_gif, d_npy = tmp_path / f"gif_{flag}", tmp_path / f"npy_{flag}"
        d_gif.mkdir()
        d_npy.mkdir()
        np.save(d_npy / "stack.npy", plane[idx].astype(np.uint8))
        for d, src in ((d_gif, gif), (d_npy, d_npy / "stack.npy")):
            r = subprocess.run([CLI, "-b", "16", "-p", "20", "-c", flag, str(src)], capture_output=True, text=True,
                               cwd=d)
            assert r.returncode == 0, r.stderr
        assert open(d_gif / "bispectrum.dat", "rb").read() == open(d_npy / "bispectrum.dat", "rb").read()
        assert np.array_equal(read_png16(d_gif / "sum_image.png"), read_png16(d_npy / "sum_image.png"))


@pytest.mark.gpu
def test_cli_apply_ignored(smip, tmp_path):
    """--apply-ignored -r 3 -k 32:16 -s 71:59: frame 3 is the correlation
    reference and every frame is cut to the 71x59 box at column 32, row 16
    (an odd size on both axes, as the reference's FFTW plans take);
    --no-calcsum drops the sum images, --no-specklemasking the bispectrum and
    everything made from it.  Outputs equal the binding on those frames."""
    _need_cli()
    from smip_gb300 import synthetic as S

    frames = S.make_stack(S.config_spec("binary128", nframes=12))
    src = tmp_path / "stack.npy"
    np.save(src, frames)
    d1, d2 = tmp_path / "a", tmp_path / "b"
    d1.mkdir()
    d2.mkdir()
    base = [CLI, "--apply-ignored", "-r", "3", "-k", "32:16", "-s", "71:59", "-b", "16", "-p", "20"]
    r = subprocess.run(base + ["--no-calcsum", str(src)], capture_output=True, text=True, cwd=d1)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(base + ["--no-specklemasking", str(src)], capture_output=True, text=True, cwd=d2)
    assert r.returncode == 0, r.stderr
    order = [3] + [i for i in range(12) if i != 3]
    used = np.ascontiguousarray(frames[order][:, 16:75, 32:103])
    with smip.Stack(71, 59, 16) as st:
        st.push_frames(used)
        ref_dat = tmp_path / "ref.dat"
        st.save_bispectrum(str(ref_dat))
        img, _, _, _ = st.finish(20.0)
        sm = st.sum()
    assert open(d1 / "bispectrum.dat", "rb").read() == open(ref_dat, "rb").read()
    assert not (d1 / "sum_image.png").exists() and not (d1 / "sum_image_falsecolor.png").exists()
    exp = np.clip(np.roll(np.abs(img), (59 // 2, 71 // 2), axis=(0, 1)) * 65535.0, 0, 65535).astype(np.uint16)
    assert np.abs(read_png16(d1 / "reco_image.png").astype(np.int64) - exp).max() <= 1
    for name in ("bispectrum.dat", "reco_image.png", "phases.png", "phasecons.png"):
        assert not (d2 / name).exists(), name
    exp = np.clip(np.abs(sm / 255.0) * 65535.0, 0, 65535).astype(np.uint16)
    assert np.abs(read_png16(d2 / "sum_image.png").astype(np.int64) - exp).max() <= 1
    assert read_png16(d2 / "powerspec.png").shape == (59, 71)
