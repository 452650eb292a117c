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
        l.ozo_decode_transform.restype = ctypes.c_int64
        l.ozo_decode_transform.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
        l.ozo_tokenize.restype = ctypes.c_int64
        l.ozo_tokenize.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        l.ozo_decompress_multi.restype = ctypes.c_int64
        l.ozo_decompress_multi.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]
        l.ozo_free.restype = None
        l.ozo_free.argtypes = [ctypes.c_void_p]
        l.ozo_test_set_fse_max_tablelog.restype = None
        l.ozo_test_set_fse_max_tablelog.argtypes = [ctypes.c_uint]
        l.ozo_test_set_huf_max_tablelog.restype = None
        l.ozo_test_set_huf_max_tablelog.argtypes = [ctypes.c_uint]
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


def decompress_multi(frame, max_outputs=64, with_lengths=False):
    """Returns [(bytes as uint8 array, type, elt_width)] per output, plus the
    string lengths (uint32 array, None for other types) with `with_lengths`;
    raises on error."""
    f = np.frombuffer(bytes(frame), np.uint8) if not isinstance(frame, np.ndarray) else frame.view(np.uint8)
    outs = (ctypes.c_void_p * max_outputs)()
    lens = (ctypes.c_size_t * max_outputs)()
    types = (ctypes.c_int * max_outputs)()
    widths = (ctypes.c_int * max_outputs)()
    slens = (ctypes.c_void_p * max_outputs)()
    nbs = (ctypes.c_size_t * max_outputs)()
    n = lib().ozo_decompress_multi(f.ctypes.data, f.size, max_outputs, outs, lens, types, widths, slens, nbs)
    if n < 0:
        raise ValueError("oracle: decode failed (%d)" % n)
    res = []
    for o in range(n):
        buf = (ctypes.c_uint8 * max(lens[o], 1)).from_address(outs[o])
        data = np.frombuffer(buf, np.uint8)[:lens[o]].copy()
        sl = None
        if types[o] == 8:
            sbuf = (ctypes.c_uint32 * max(nbs[o], 1)).from_address(slens[o])
            sl = np.frombuffer(sbuf, np.uint32)[:nbs[o]].copy()
        lib().ozo_free(outs[o])
        lib().ozo_free(slens[o])
        res.append((data, types[o], widths[o], sl) if with_lengths else (data, types[o], widths[o]))
    return res


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


def compress_tablelog12(recipe, arr, elt_width, checksums=True):
    """Like compress(), but the FSE encoder may pick table log 12 (the
    decoders' limit) where the reference's encoder stops at 11. Test frames
    for the widest FSE fields; valid for the reference's decoder."""
    lib().ozo_test_set_fse_max_tablelog(12)
    try:
        return compress(recipe, arr, elt_width, checksums)
    finally:
        lib().ozo_test_set_fse_max_tablelog(11)


def compress_huf_tablelog12(recipe, arr, elt_width, checksums=True):
    """Like compress(), but the Huffman encoder may pick table log 12 (the
    decoders' limit) where the reference's encoder stops at 11. Test frames
    for the widest Huffman tables; valid for the reference's decoder."""
    lib().ozo_test_set_huf_max_tablelog(12)
    try:
        return compress(recipe, arr, elt_width, checksums)
    finally:
        lib().ozo_test_set_huf_max_tablelog(11)


def xxh3_64(buf):
    b = np.frombuffer(bytes(buf), np.uint8)
    return lib().ozo_xxh3_64(b.ctypes.data, b.size)


TYPE_SERIAL, TYPE_STRUCT, TYPE_NUMERIC = 1, 2, 4


def decode_transform(trid, header, inputs, out_cap=1 << 20):
    """One decoder on explicit streams: inputs = [(type, width, bytes)] in the
    decoder's order. Returns (output bytes, type, width, count)."""
    n = len(inputs)
    bufs = [np.frombuffer(bytes(b), np.uint8).copy() if len(b) else np.zeros(1, np.uint8) for _, _, b in inputs]
    types = (ctypes.c_int * max(n, 1))(*[t for t, _, _ in inputs])
    widths = (ctypes.c_size_t * max(n, 1))(*[w for _, w, _ in inputs])
    counts = (ctypes.c_size_t * max(n, 1))(*[len(b) // w for _, w, b in inputs])
    ptrs = (ctypes.c_void_p * max(n, 1))(*[b.ctypes.data for b in bufs])
    h = np.frombuffer(bytes(header), np.uint8).copy() if header else np.zeros(1, np.uint8)
    out = np.empty(out_cap, np.uint8)
    t, w, c = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t()
    r = lib().ozo_decode_transform(trid, h.ctypes.data, len(header), n, types, widths, counts, ptrs, out.ctypes.data,
                                   out_cap, ctypes.byref(t), ctypes.byref(w), ctypes.byref(c))
    if r < 0:
        raise ValueError("oracle: decoder failed (%d)" % r)
    return out[:r].copy(), t.value, w.value, c.value


def tokenize(arr, sorted_alphabet=False):
    """The tokenize node alone: (alphabet array, indices array)."""
    a = np.ascontiguousarray(arr)
    alpha = np.empty(max(a.size, 1), a.dtype)
    idx = np.empty(max(a.size, 1) * 4, np.uint8)
    iw = ctypes.c_int()
    na = lib().ozo_tokenize(a.ctypes.data, a.size, a.itemsize, 1 if sorted_alphabet else 0, alpha.ctypes.data,
                            idx.ctypes.data, ctypes.byref(iw))
    dt = {1: np.uint8, 2: np.uint16, 4: np.uint32}[iw.value]
    return alpha[:na].copy(), idx[: a.size * iw.value].view(dt).copy()

