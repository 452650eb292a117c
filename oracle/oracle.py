"""ctypes bindings of the CPU oracle (oracle/_build/libozl_oracle.so).

Test infrastructure only: imported by the tests, the smoke check and the
benchmark's CPU-baseline leg, never by the openzl_gb300 package.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libozl_oracle.so")
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-f", os.path.join("oracle", "Makefile")], cwd=ROOT)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        l = ctypes.CDLL(LIB)
        l.ozo_decompress.restype = ctypes.c_int64
        l.ozo_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        l.ozo_decompressed_size.restype = ctypes.c_int64
        l.ozo_decompressed_size.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        l.ozo_compress.restype = ctypes.c_int64
        l.ozo_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        l.ozo_compress_bound.restype = ctypes.c_size_t
        l.ozo_compress_bound.argtypes = [ctypes.c_size_t]
        l.ozo_xxh3_64.restype = ctypes.c_uint64
        l.ozo_xxh3_64.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        _lib = l
    return _lib


def decompress(frame):
    """Returns (bytes as uint8 array, type, elt_width); raises on error."""
    f = np.frombuffer(bytes(frame), np.uint8) if not isinstance(frame, np.ndarray) else frame.view(np.uint8)
    n = lib().ozo_decompressed_size(f.ctypes.data, f.size)
    if n < 0:
        raise ValueError("oracle: bad frame (%d)" % n)
    out = np.empty(max(int(n), 1) + 16, np.uint8)
    t, w = ctypes.c_int(), ctypes.c_int()
    r = lib().ozo_decompress(f.ctypes.data, f.size, out.ctypes.data, out.size, ctypes.byref(t), ctypes.byref(w))
    if r < 0:
        raise ValueError("oracle: decode failed (%d)" % r)
    return out[:r], t.value, w.value


def compress(recipe, arr, elt_width, checksums=True):
    arr = np.ascontiguousarray(arr)
    n = arr.size if elt_width else arr.nbytes
    cap = lib().ozo_compress_bound(arr.nbytes)
    dst = np.empty(cap, np.uint8)
    r = lib().ozo_compress(recipe, arr.ctypes.data if arr.size else None, n, elt_width, dst.ctypes.data, cap,
                           1 if checksums else 0)
    if r < 0:
        raise ValueError("oracle: compress failed (%d)" % r)
    return dst[:r].copy()


def xxh3_64(buf):
    b = np.frombuffer(bytes(buf), np.uint8)
    return lib().ozo_xxh3_64(b.ctypes.data, b.size)
