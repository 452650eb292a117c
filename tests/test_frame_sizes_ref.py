"""Frame-size entry points against the reference's own library (built here
by oracle/ref.mk; skipped where it is absent): ZL_getDecompressedSize agrees
with the reference on success or failure and on the value for every golden
frame and 40 mutated copies of each (bytes flipped or replaced, frames cut);
ZL_getCompressedSize agrees on every golden frame."""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libozl_ref.so")
pytestmark = pytest.mark.skipif(not os.path.exists(REF_LIB), reason="the reference oracle (oracle/_ref) is not built here")


class _Report(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("value", ctypes.c_size_t)]


def _libs():
    from openzl_gb300 import _lib

    ours = ctypes.CDLL(_lib.library_path())
    ref = ctypes.CDLL(REF_LIB)
    for lib in (ours, ref):
        for fn in ("ZL_getDecompressedSize", "ZL_getCompressedSize"):
            f = getattr(lib, fn)
            f.restype = _Report
            f.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    return ours, ref


def _same(a, b):
    return (a.code != 0) == (b.code != 0) and (a.code != 0 or a.value == b.value)


def test_frame_sizes_match_reference():
    ours, ref = _libs()
    rng = np.random.default_rng(31)
    bad = []
    for path in sorted(glob.glob(os.path.join(GOLDEN, "*.zl"))):
        frame = np.fromfile(path, np.uint8)
        for fn in ("ZL_getDecompressedSize", "ZL_getCompressedSize"):
            a = getattr(ours, fn)(frame.ctypes.data, frame.size)
            b = getattr(ref, fn)(frame.ctypes.data, frame.size)
            if not _same(a, b):
                bad.append((os.path.basename(path), fn, a.code, a.value, b.code, b.value))
        for k in range(40):
            m = frame.copy()
            at = int(rng.integers(0, max(1, min(m.size, 48) if k % 2 else m.size)))
            kind = k % 3
            if kind == 0:
                m[at] ^= np.uint8(1 << int(rng.integers(0, 8)))
            elif kind == 1:
                m[at] = np.uint8(rng.integers(0, 256))
            else:
                m = np.ascontiguousarray(m[:at])
            p = m.ctypes.data if m.size else None
            a = ours.ZL_getDecompressedSize(p, m.size)
            b = ref.ZL_getDecompressedSize(p, m.size)
            if not _same(a, b):
                bad.append((os.path.basename(path), k, a.code, a.value, b.code, b.value))
    assert not bad, bad[:10]
