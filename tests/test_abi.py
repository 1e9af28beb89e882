"""C-ABI boundary without a GPU: the library loads, exports every symbol that
include/smip_gpu.h declares, and its host-side logic (spiral visits,
argument validation) behaves like the reference."""
import ctypes as C
import hashlib
import os
import re

import numpy as np
import pytest
from conftest import ROOT, golden


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "smip_gpu.h")).read()
    return sorted(set(re.findall(r"SMIP_GPU_API\s+[\w\s\*]+?\b(smip_\w+)\s*\(", src)))


def test_exports_every_declared_symbol(smip):
    names = declared_symbols()
    assert len(names) >= 20
    lib = C.CDLL(smip.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version(smip):
    assert smip.version() == (0, 3, 2)


def test_next_reco_index_and_visits(smip):
    assert smip.next_reco_index(0.0, 0.0, 0, 0) == (1.0, 0.0, 1, 0)
    fx = golden("reco_visits")
    for R in (12, 64, 128, 200):
        v = smip.reco_visits(R)
        assert len(v) == int(fx[f"r{R}_count"])
        assert hashlib.sha256(v.astype(np.int32).tobytes()).hexdigest() == str(fx[f"r{R}_sha"])


@pytest.mark.parametrize("shape", [(128, 128, 66), (128, 128, 1), (128, 128, 128), (4, 100, 4), (2, 64, 2),
                                   (1025, 64, 8), (64, 2048, 8), (16, 16, 16)])
def test_unsupported_shapes_rejected(smip, shape):
    """Depths outside [2, 64] or not below the frame, and sides outside
    [3, 1024], are refused before any device work."""
    with pytest.raises(smip.Unsupported):
        smip.Stack(*shape)


def test_window_domain_error(smip):
    with pytest.raises(smip.DomainError):
        smip.hann(16, 16, 0.0)


def test_base_size(smip):
    assert smip.bispec_base_size(256, 256, 32) == 18598833
    assert smip.bispec_base_size(512, 512, 48) == 161505225
    assert smip.bispec_base_size(128, 128, 33) == smip.bispec_base_size(128, 128, 32)
    from oracle import bispec_desc

    for W, H, D in ((99, 75, 14), (100, 100, 20), (640, 480, 16), (37, 64, 8)):  # any frame size
        assert smip.bispec_base_size(W, H, D) == bispec_desc(W, H, D)["base_size"]
