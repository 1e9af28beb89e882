"""smip-cli's SER and AVI readers (cli/video_decode.hpp) on files written here.

The reference takes video through OpenCV's VideoCapture (videoio.cpp:13-52),
which hands frames over as 8-bit BGR images.  The readers are checked
against the frames the test wrote: mono and colour SER (8 and 16 bits, both
byte orders), AVI with 24- and 32-bit BGR rows (bottom-up and top-down, with
row padding), an 8-bit colour table, Y800 and Y16 gray, a dropped frame and an
OpenDML "AVIX" extension.  The GPU test runs smip-cli on a SER file and on the
same frames as .npy and requires identical outputs.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "speckle-stacker_gb300")
CLI = os.path.join(PKG, "bin", "smip-cli")


@pytest.fixture(scope="module")
def video_check(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ missing")
    exe = str(tmp_path_factory.mktemp("vc") / "video_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(PKG, "cli"),
                    os.path.join(ROOT, "tests", "cpp", "video_check.cpp"), "-o", exe], check=True)
    return exe


def decode(exe, path, tmp_path):
    raw = str(tmp_path / "frames.raw")
    r = subprocess.run([exe, str(path), raw], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n, h, w, ch, es = (int(x) for x in r.stdout.split())
    a = np.fromfile(raw, np.uint8 if es == 1 else np.uint16)
    return a.reshape((n, h, w, ch) if ch > 1 else (n, h, w))


# ------------------------------------------------------------------ writers
def write_ser(path, frames, color_id=0, little=1, depth=None, big_endian_data=False, nframes_field=None):
    """SER v3: 178-byte header, then the frames (planes interleaved per pixel)."""
    n, h, w = frames.shape[:3]
    depth = depth or (8 if frames.dtype == np.uint8 else 16)
    hdr = b"LUCAM-RECORDER" + struct.pack("<iiiiiii", 0, color_id, little, w, h, depth,
                                          n if nframes_field is None else nframes_field)
    hdr += b"observer".ljust(40, b"\0") + b"instrument".ljust(40, b"\0") + b"telescope".ljust(40, b"\0")
    hdr += struct.pack("<qq", 0, 0)
    assert len(hdr) == 178
    data = frames.astype(">u2" if big_endian_data else "<u2").tobytes() if frames.dtype == np.uint16 else frames.tobytes()
    with open(path, "wb") as f:
        f.write(hdr + data + b"TRAILER-TIMESTAMPS")


def _chunk(cid, body):
    return cid + struct.pack("<I", len(body)) + body + (b"\0" if len(body) & 1 else b"")


def _list(ltype, body):
    return b"LIST" + struct.pack("<I", len(body) + 4) + ltype + body


def write_avi(path, stored_frames, w, h, bits, comp=0, palette=None, extra_streams=False, split=None):
    """Uncompressed AVI; stored_frames are the chunk bodies (already laid out)."""
    bih = struct.pack("<IiiHHIIiiII", 40, w, h, 1, bits, comp, 0, 0, 0, 0, 0)
    if palette is not None:
        bih += palette.tobytes()
    strls = b""
    if extra_streams:  # an audio stream first: the video stream is then 01
        strls += _list(b"strl", _chunk(b"strh", b"auds" + b"\0" * 52) + _chunk(b"strf", b"\0" * 18))
    strls += _list(b"strl", _chunk(b"strh", b"vids" + b"DIB " + b"\0" * 48) + _chunk(b"strf", bih))
    avih = struct.pack("<IIIIIIIIII", 40000, 0, 0, 0, len(stored_frames), 0, 1, 0, w, abs(h)) + b"\0" * 16
    hdrl = _list(b"hdrl", _chunk(b"avih", avih) + strls)
    sid = b"01" if extra_streams else b"00"
    first = stored_frames if split is None else stored_frames[:split]
    movi = _list(b"movi", b"".join(_chunk(sid + b"db", fr) for fr in first))
    body = b"AVI " + hdrl + movi + _chunk(b"idx1", b"")
    out = b"RIFF" + struct.pack("<I", len(body)) + body
    if split is not None:  # OpenDML: the remaining frames in a RIFF AVIX
        movi2 = _list(b"movi", b"".join(_chunk(sid + b"db", fr) for fr in stored_frames[split:]))
        body2 = b"AVIX" + movi2
        out += b"RIFF" + struct.pack("<I", len(body2)) + body2
    with open(path, "wb") as f:
        f.write(out)


def bgr_rows(frame_bgr, bits, bottom_up):
    h, w, _ = frame_bgr.shape
    px = frame_bgr if bits == 24 else np.concatenate([frame_bgr, np.full((h, w, 1), 77, np.uint8)], axis=2)
    rows = px.reshape(h, -1)
    stride = (w * bits // 8 + 3) // 4 * 4
    pad = np.zeros((h, stride - rows.shape[1]), np.uint8)
    rows = np.concatenate([rows, pad], axis=1)
    return (rows[::-1] if bottom_up else rows).tobytes()


# ------------------------------------------------------------------- tests
def test_ser_mono8_and_truncated(video_check, tmp_path):
    rng = np.random.default_rng(1)
    fr = rng.integers(0, 256, (5, 24, 40), dtype=np.uint8)
    write_ser(tmp_path / "a.ser", fr)
    assert np.array_equal(decode(video_check, tmp_path / "a.ser", tmp_path), fr)
    # a header that claims more frames than the file holds keeps the whole ones
    write_ser(tmp_path / "b.ser", fr, nframes_field=9)
    assert np.array_equal(decode(video_check, tmp_path / "b.ser", tmp_path), fr)


@pytest.mark.parametrize("little,big_data", [(1, False), (0, True)])
def test_ser_mono16_byte_orders(video_check, tmp_path, little, big_data):
    rng = np.random.default_rng(2)
    fr = rng.integers(0, 65536, (4, 16, 20), dtype=np.uint16)
    write_ser(tmp_path / "c.ser", fr, little=little, depth=16, big_endian_data=big_data)
    assert np.array_equal(decode(video_check, tmp_path / "c.ser", tmp_path), fr)


def test_ser_12bit_and_bayer_as_one_channel(video_check, tmp_path):
    rng = np.random.default_rng(3)
    fr = rng.integers(0, 4096, (3, 8, 12), dtype=np.uint16)
    write_ser(tmp_path / "d.ser", fr, color_id=8, depth=12)  # RGGB mosaic, 12-bit samples in 2 bytes
    assert np.array_equal(decode(video_check, tmp_path / "d.ser", tmp_path), fr)


@pytest.mark.parametrize("color_id", [100, 101])
def test_ser_colour_delivered_bgr(video_check, tmp_path, color_id):
    rng = np.random.default_rng(4)
    fr = rng.integers(0, 256, (3, 10, 14, 3), dtype=np.uint8)
    write_ser(tmp_path / "e.ser", fr, color_id=color_id)
    got = decode(video_check, tmp_path / "e.ser", tmp_path)
    exp = fr[..., ::-1] if color_id == 100 else fr  # RGB planes come out as B, G, R
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("bits,bottom_up,w", [(24, True, 13), (24, False, 16), (32, True, 7)])
def test_avi_bgr(video_check, tmp_path, bits, bottom_up, w):
    rng = np.random.default_rng(bits + w)
    h = 9
    fr = rng.integers(0, 256, (4, h, w, 3), dtype=np.uint8)
    write_avi(tmp_path / "a.avi", [bgr_rows(f, bits, bottom_up) for f in fr], w, h if bottom_up else -h, bits)
    assert np.array_equal(decode(video_check, tmp_path / "a.avi", tmp_path), fr)


def test_avi_palette_and_second_stream(video_check, tmp_path):
    rng = np.random.default_rng(5)
    h, w = 6, 10
    pal = np.zeros((256, 4), np.uint8)
    pal[:, 0] = np.arange(256)            # B
    pal[:, 1] = 255 - np.arange(256)      # G
    pal[:, 2] = (np.arange(256) * 3) % 256  # R
    idx = rng.integers(0, 256, (3, h, w), dtype=np.uint8)
    stored = []
    for f in idx:
        rows = np.concatenate([f, np.zeros((h, 2), np.uint8)], axis=1)  # stride 12
        stored.append(rows[::-1].tobytes())
    write_avi(tmp_path / "p.avi", stored, w, h, 8, palette=pal, extra_streams=True)
    got = decode(video_check, tmp_path / "p.avi", tmp_path)
    assert np.array_equal(got, pal[idx][..., :3])


def test_avi_gray_dropped_frame_and_avix(video_check, tmp_path):
    rng = np.random.default_rng(6)
    h, w = 5, 11
    fr = rng.integers(0, 256, (6, h, w), dtype=np.uint8)
    stored = [f.tobytes() for f in fr]
    stored[3] = b""  # dropped: repeats frame 2
    y800 = struct.unpack("<I", b"Y800")[0]
    write_avi(tmp_path / "g.avi", stored, w, h, 8, comp=y800, split=4)
    got = decode(video_check, tmp_path / "g.avi", tmp_path)
    exp = fr.copy()
    exp[3] = fr[2]
    assert np.array_equal(got, exp)


def test_avi_y16(video_check, tmp_path):
    rng = np.random.default_rng(7)
    fr = rng.integers(0, 65536, (3, 4, 6), dtype=np.uint16)
    y16 = struct.unpack("<I", b"Y16 ")[0]
    write_avi(tmp_path / "y.avi", [f.astype("<u2").tobytes() for f in fr], 6, 4, 16, comp=y16)
    assert np.array_equal(decode(video_check, tmp_path / "y.avi", tmp_path), fr)


def test_avi_compressed_refused(video_check, tmp_path):
    mjpg = struct.unpack("<I", b"MJPG")[0]
    write_avi(tmp_path / "m.avi", [b"\xff\xd8junk"], 8, 8, 24, comp=mjpg)
    r = subprocess.run([video_check, str(tmp_path / "m.avi"), str(tmp_path / "x.raw")], capture_output=True, text=True)
    assert r.returncode == 1 and "unsupported AVI video format" in r.stderr


@pytest.mark.gpu
def test_cli_ser_matches_npy(tmp_path):
    """smip-cli on a 16-bit SER file gives byte-identical outputs to the same
    frames as a .npy stack."""
    if not os.path.exists(CLI):
        pytest.skip("smip-cli not built")
    import sys

    sys.path.insert(0, PKG)
    from smip_gb300 import synthetic as S

    frames = S.make_stack(S.config_spec("extended256", n=64, nframes=24, bdepth=16, reco_radius=24))
    a, b = tmp_path / "ser", tmp_path / "npy"
    a.mkdir()
    b.mkdir()
    write_ser(a / "stack.ser", frames, depth=16)
    np.save(b / "stack.npy", frames)
    for d, name in ((a, "stack.ser"), (b, "stack.npy")):
        r = subprocess.run([CLI, "-b", "16", "-p", "24", name], capture_output=True, text=True, cwd=d)
        assert r.returncode == 0, r.stderr
    for name in sorted(os.listdir(b)):
        if name.endswith(".png") or name == "bispectrum.dat":
            assert open(a / name, "rb").read() == open(b / name, "rb").read(), name
