"""smip-cli's GIF input (speckle-stacker_gb300/cli/gif_decode.hpp): frames
composed on the logical screen in BGR order, as OpenCV's VideoCapture delivers
them to the reference's Mat2Array (include/videoio.h:71-98).

The GIFs here are written by a small LZW encoder in this file: full frames
with local colour tables, a sub-rectangle with a transparent index, an
interlaced frame, and the three disposal methods; random images long enough to
reach 12-bit codes and table resets."""
import os
import shutil
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "speckle-stacker_gb300", "cli")


def lzw_encode(idx, min_code):
    """GIF LZW: codes of width min_code+1 growing to 12 bits, a clear code at
    the start and whenever the 4096-entry table is full, then the end code."""
    clear, eoi = 1 << min_code, (1 << min_code) + 1
    out, acc, nacc = bytearray(), 0, 0

    def emit(code, width):
        nonlocal acc, nacc
        acc |= code << nacc
        nacc += width
        while nacc >= 8:
            out.append(acc & 0xFF)
            acc >>= 8
            nacc -= 8

    def reset():
        return {(i,): i for i in range(clear)}, eoi + 1, min_code + 1

    table, nxt, width = reset()
    emit(clear, width)
    w = ()
    for k in idx:
        wk = w + (int(k),)
        if wk in table:
            w = wk
            continue
        emit(table[w], width)
        table[wk] = nxt
        nxt += 1
        if nxt - 1 == (1 << width) and width < 12:
            width += 1
        if nxt == 4096:
            emit(clear, width)
            table, nxt, width = reset()
        w = (int(k),)
    if w:
        emit(table[w], width)
    emit(eoi, width)
    if nacc:
        out.append(acc & 0xFF)
    return bytes(out)


def sub_blocks(b):
    return b"".join(bytes([len(b[i:i + 255])]) + b[i:i + 255] for i in range(0, len(b), 255)) + b"\0"


def write_gif(path, W, H, frames, gct=None, bg=0):
    """frames: dicts with idx (h x w), left, top, lct (n x 3 RGB or None),
    interlace, transparent (index or None), disposal."""
    with open(path, "wb") as f:
        gbits = 0
        if gct is not None:
            gbits = 0x80 | (int(np.log2(len(gct))) - 1)
        f.write(b"GIF89a" + struct.pack("<HHBBB", W, H, gbits, bg, 0))
        if gct is not None:
            f.write(np.asarray(gct, np.uint8).tobytes())
        for fr in frames:
            tr = fr.get("transparent")
            f.write(b"\x21\xF9\x04" + bytes([(fr.get("disposal", 0) << 2) | (1 if tr is not None else 0)])
                    + b"\0\0" + bytes([tr or 0]) + b"\0")
            h, w = fr["idx"].shape
            lct = fr.get("lct")
            ibits = (0x80 | (int(np.log2(len(lct))) - 1)) if lct is not None else 0
            if fr.get("interlace"):
                ibits |= 0x40
            f.write(b"\x2C" + struct.pack("<HHHHB", fr.get("left", 0), fr.get("top", 0), w, h, ibits))
            if lct is not None:
                f.write(np.asarray(lct, np.uint8).tobytes())
            rows = fr["idx"]
            if fr.get("interlace"):
                order = list(range(0, h, 8)) + list(range(4, h, 8)) + list(range(2, h, 4)) + list(range(1, h, 2))
                rows = rows[order]
            f.write(bytes([8]) + sub_blocks(lzw_encode(rows.ravel(), 8)))
        f.write(b"\x3B")


def compose(W, H, frames, gct, bg):
    """Reference composition (BGR), the rules gif_decode.hpp states."""
    canvas = np.zeros((H, W, 3), np.uint8)
    out = []
    for fr in frames:
        ct = np.asarray(fr["lct"] if fr.get("lct") is not None else gct, np.uint8)
        saved = canvas.copy()
        h, w = fr["idx"].shape
        l, t = fr.get("left", 0), fr.get("top", 0)
        for y in range(h):
            for x in range(w):
                c = fr["idx"][y, x]
                if fr.get("transparent") is not None and c == fr["transparent"]:
                    continue
                if t + y < H and l + x < W:
                    canvas[t + y, l + x] = ct[c][::-1]
        out.append(canvas.copy())
        d = fr.get("disposal", 0)
        if d == 2:  # the background colour of the global table, black without one or when transparent
            col = np.zeros(3, np.uint8)
            if gct is not None and fr.get("transparent") is None:
                col = np.asarray(gct, np.uint8)[bg][::-1]
            canvas[t:t + h, l:l + w] = col
        elif d == 3:
            canvas = saved
    return np.stack(out)


@pytest.fixture(scope="module")
def gif_check(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("gif") / "gif_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", CLI,
                    os.path.join(ROOT, "tests", "cpp", "gif_check.cpp"), "-o", exe], check=True)
    return exe


def decode(exe, path, tmp_path):
    raw = str(tmp_path / "frames.raw")
    r = subprocess.run([exe, path, raw], capture_output=True, text=True, check=True)
    n, h, w = map(int, r.stdout.split())
    return np.fromfile(raw, np.uint8).reshape(n, h, w, 3)


def test_composition_and_lzw(gif_check, tmp_path):
    rng = np.random.default_rng(3)
    W, H = 48, 40
    gct = rng.integers(0, 256, (256, 3))
    lct = rng.integers(0, 256, (256, 3))
    frames = [
        {"idx": rng.integers(0, 256, (H, W)), "lct": lct, "disposal": 1},           # full frame, local table
        {"idx": rng.integers(0, 4, (10, 20)), "left": 5, "top": 7, "transparent": 2,  # sub-rectangle
         "disposal": 2},
        {"idx": (np.arange(30 * 17).reshape(30, 17) % 7), "left": 20, "top": 3,      # long runs: multi-code strings
         "interlace": True, "disposal": 3},
        {"idx": rng.integers(0, 256, (H, W))},                                        # after a restore-previous
    ]
    path = str(tmp_path / "t.gif")
    write_gif(path, W, H, frames, gct=gct, bg=9)
    got = decode(gif_check, path, tmp_path)
    exp = compose(W, H, frames, gct, 9)
    assert got.shape == exp.shape
    assert np.array_equal(got, exp)


def test_long_random_image_reaches_12_bit_codes(gif_check, tmp_path):
    rng = np.random.default_rng(4)
    W, H = 200, 150  # 30,000 random pixels: the table fills and resets several times
    gct = rng.integers(0, 256, (256, 3))
    frames = [{"idx": rng.integers(0, 256, (H, W))}, {"idx": np.zeros((H, W), int) + 17}]
    path = str(tmp_path / "big.gif")
    write_gif(path, W, H, frames, gct=gct)
    got = decode(gif_check, path, tmp_path)
    assert np.array_equal(got, compose(W, H, frames, gct, 0))


def test_reference_testdata_gif_decodes(gif_check, tmp_path):
    """The reference's own sample stack (data/testdata.gif, read by smip-cli
    through OpenCV): 40 frames of 128x128 decode to a speckle cloud brighter
    in the centre than at the edges."""
    from oracle import REFERENCE

    ref = os.path.join(REFERENCE, "data", "testdata.gif")
    if not os.path.exists(ref):
        pytest.skip("reference data not present")
    got = decode(gif_check, ref, tmp_path)
    assert got.shape == (40, 128, 128, 3)
    m = got[..., 2].astype(float).mean(axis=0)
    assert m[56:72, 56:72].mean() > 2 * m[:8, :8].mean()


def read_png_any(path):
    """8/16-bit gray or RGB PNG with any of the five row filters (the
    reference's published images are written by OpenCV); first channel."""
    data = open(path, "rb").read()
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype = ihdr[:4]
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    bpp = ch * depth // 8
    stride = w * bpp
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, stride + 1)
    out = np.zeros((h, stride), np.int64)
    prev = np.zeros(stride, np.int64)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int64)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 0xFF
        else:  # Sub, Average and Paeth depend on the pixel to the left: byte by byte
            cur = np.zeros(stride, np.int64)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b, c = prev[x], (prev[x - bpp] if x >= bpp else 0)
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) // 2
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 0xFF
        out[y] = cur
        prev = cur
    px = out.astype(np.uint8)
    px = px.view(">u2").astype(np.uint16) if depth == 16 else px
    return px.reshape(h, w, ch)[..., 0]


def _ncc(a, b):
    a = a.astype(float).ravel() - a.mean()
    b = b.astype(float).ravel() - b.mean()
    return float((a * b).sum() / np.sqrt((a * a).sum() * (b * b).sum()))


def test_reference_example_matches_published_images(gif_check, oracle, tmp_path):
    """The reference's worked example (README: `smip-cli -v -b 32 -p 64 -c r
    data/hu940ani/hu940ani.gif`, 40 frames of the binary star HU 940) through
    this decoder and the oracle's pipeline, mapped to 16 bits as
    smip-cli/main.cpp:359-388 does, against the PNGs the reference publishes
    beside the GIF.  Those images were made by OpenCV's GIF reader, not this
    decoder, so they are compared by correlation: the reconstruction agrees at
    ncc 0.991, the shift-and-add sum at 0.984 once offset by one pixel in x."""
    from oracle import REFERENCE

    d = os.path.join(REFERENCE, "data", "hu940ani")
    if not os.path.exists(os.path.join(d, "hu940ani.gif")):
        pytest.skip("reference data not present")
    frames = decode(gif_check, os.path.join(d, "hu940ani.gif"), tmp_path)
    # -c r: channel round(log2(1)) = 0 of B, G, R (videoio.h:78-79); B equals R in this GIF
    red = np.ascontiguousarray(frames[..., 0])
    n, H, W = red.shape
    out = oracle.run_stack(red, 32, 64)

    def to16(v):
        s = v * 65535.0
        return np.where(s >= 65535.0, 65535.0, np.where(s > 0.0, s, 0.0)).astype(np.uint16)

    reco = to16(np.roll(np.abs(out["image"]), (H // 2, W // 2), (0, 1)))
    sum16 = to16(np.abs(out["sum"]) / 255.0)
    ref_reco = read_png_any(os.path.join(d, "reco_image.png"))
    ref_sum = read_png_any(os.path.join(d, "sum_image.png"))
    assert reco.shape == ref_reco.shape == (128, 128)
    assert reco.max() == ref_reco.max() == 65535  # both max-normalised
    assert _ncc(reco, ref_reco) > 0.985
    best = max(_ncc(np.roll(sum16, (dy, dx), (0, 1)), ref_sum) for dy in (-1, 0, 1) for dx in (-1, 0, 1))
    assert best > 0.975
    assert abs(sum16.mean() / ref_sum.mean() - 1.0) < 0.01
