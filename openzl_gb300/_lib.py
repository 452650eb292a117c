"""ctypes bindings of libopenzl_gb300 (names and semantics of include/openzl_gb300.h)."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libopenzl_gb300.so")
_lib = None


class ZLReport(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("value", ctypes.c_size_t)]


class ZLError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("openzl_gb300 error %d: %s" % (code, msg))
        self.code = code


def library_path():
    return _LIB_PATH


def library():
    """Loads the compiled library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise ZLError(1, "libopenzl_gb300.so is not built (run openzl_gb300.build.build())")
    lib = ctypes.CDLL(_LIB_PATH)
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    sig = {
        "ZL_getDecompressedSize": ([vp, sz], ZLReport),
        "ZL_getCompressedSize": ([vp, sz], ZLReport),
        "ZL_DCtx_create": ([], vp),
        "ZL_DCtx_free": ([vp], None),
        "ZL_DCtx_setParameter": ([vp, ctypes.c_int, ctypes.c_int], ZLReport),
        "ZL_DCtx_getErrorContextString": ([vp, ZLReport], ctypes.c_char_p),
        "ZL_DCtx_decompress": ([vp, vp, sz, vp, sz], ZLReport),
        "ZL_decompress": ([vp, sz, vp, sz], ZLReport),
        "ZL_ErrorCode_toString": ([ctypes.c_int], ctypes.c_char_p),
        "ozl_gpu_decompress": ([vp, vp, sz, vp, vp, sz, vp], ZLReport),
        "ozl_gpu_batch_create": ([], vp),
        "ozl_gpu_batch_free": ([vp], None),
        "ozl_gpu_batch_setParameter": ([vp, ctypes.c_int, ctypes.c_int], ZLReport),
        "ozl_gpu_batch_plan": ([vp, sz, vp, vp, vp, vp, vp], ZLReport),
        "ozl_gpu_batch_run": ([vp, vp, ctypes.c_int], ZLReport),
        "ozl_gpu_batch_check": ([vp, vp], ZLReport),
        "ozl_gpu_batch_launches": ([vp], sz),
        "ozl_gpu_batch_sizes": ([vp], ctypes.POINTER(ctypes.c_size_t)),
        "ozl_gpu_batch_error": ([vp], ctypes.c_char_p),
        "ozl_gpu_version": ([], ctypes.c_char_p),
        "ozl_gpu_xxh3_64": ([vp, sz, vp], ZLReport),
        "ozl_gpu_xxh3_64_static": ([vp, sz, vp], ZLReport),
        "ozl_gpu_batch_profile": ([vp, vp, vp, vp, vp, sz], ZLReport),
        "ozl_gpu_kind_name": ([ctypes.c_int], ctypes.c_char_p),
        "ozl_gpu_batch_run_host": ([vp, vp, sz, vp, sz, vp, ctypes.c_int], ZLReport),
        "ozl_gpu_encoder_create": ([], vp),
        "ozl_gpu_encoder_free": ([vp], None),
        "ozl_gpu_compress_bound": ([sz], sz),
        "ozl_gpu_compress_batch": ([vp, sz, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, vp], ZLReport),
        "ozl_gpu_encoder_error": ([vp], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _check(rep, ctx_msg=""):
    if rep.code != 0:
        msg = library().ZL_ErrorCode_toString(rep.code).decode()
        raise ZLError(rep.code, msg + (": " + ctx_msg if ctx_msg else ""))
    return rep.value


def _as_u8(buf):
    if isinstance(buf, np.ndarray):
        return np.ascontiguousarray(buf).view(np.uint8).reshape(-1)
    return np.frombuffer(bytes(buf), np.uint8)


def get_decompressed_size(frame):
    f = _as_u8(frame)
    return _check(library().ZL_getDecompressedSize(f.ctypes.data, f.size))


def get_compressed_size(frame):
    f = _as_u8(frame)
    return _check(library().ZL_getCompressedSize(f.ctypes.data, f.size))


# DParam values (include/openzl_gb300.h)
DPARAM_STICKY = 1
DPARAM_CHECK_COMPRESSED = 2
DPARAM_CHECK_CONTENT = 3


class DCtx:
    """ZL_DCtx: decompression context (one per host thread)."""

    def __init__(self):
        self._lib = library()
        self._h = self._lib.ZL_DCtx_create()
        if not self._h:
            raise ZLError(70, "ZL_DCtx_create failed")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ZL_DCtx_free(h)
            self._h = None

    def set_parameter(self, param, value):
        _check(self._lib.ZL_DCtx_setParameter(self._h, param, value))

    def _err(self, rep):
        return self._lib.ZL_DCtx_getErrorContextString(self._h, rep).decode()

    def decompress(self, frame, out=None):
        """Host frame in, host bytes out (numpy uint8)."""
        f = _as_u8(frame)
        n = get_decompressed_size(f)
        if out is None:
            out = np.empty(max(n, 1), np.uint8)
        rep = self._lib.ZL_DCtx_decompress(self._h, out.ctypes.data, out.nbytes, f.ctypes.data, f.size)
        if rep.code:
            raise ZLError(rep.code, self._err(rep))
        return out[: rep.value]

    def decompress_device(self, frame_host, frame_dev_ptr, dst_dev_ptr, dst_capacity, stream=0):
        f = _as_u8(frame_host)
        rep = self._lib.ozl_gpu_decompress(self._h, dst_dev_ptr, dst_capacity, f.ctypes.data, frame_dev_ptr,
                                           f.size, stream)
        if rep.code:
            raise ZLError(rep.code, self._err(rep))
        return rep.value


def xxh3_64_device(dev_ptr, length, stream=0):
    """XXH3-64 of device memory, computed on the GPU."""
    return _check(library().ozl_gpu_xxh3_64(dev_ptr, length, stream))


XXH3_STATIC_MAX_LEN = 32 << 20


def xxh3_64_device_static(dev_ptr, length, stream=0):
    """XXH3-64 of device memory through the allocation-free entry point
    (fixed device scratch shared by all calls; at most XXH3_STATIC_MAX_LEN
    bytes; calls that overlap on the GPU race)."""
    rep = library().ozl_gpu_xxh3_64_static(dev_ptr, length, stream)
    _check(rep)
    return rep.value


def decompress(frame):
    return DCtx().decompress(frame)


class GpuBatch:
    """Batched decode of many frames: one plan, one CUDA graph per run."""

    def __init__(self, check_content=True, check_compressed=True):
        self._lib = library()
        self._h = self._lib.ozl_gpu_batch_create()
        if not check_content:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_CHECK_CONTENT, 2))
        if not check_compressed:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_CHECK_COMPRESSED, 2))
        self._keep = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ozl_gpu_batch_free(h)
            self._h = None

    def _raise(self, rep):
        raise ZLError(rep.code, self._lib.ozl_gpu_batch_error(self._h).decode())

    def plan(self, frames_host, frames_dev_ptrs, dst_dev_ptrs, dst_capacities):
        n = len(frames_host)
        hs = [_as_u8(f) for f in frames_host]
        hp = (ctypes.c_void_p * n)(*[h.ctypes.data for h in hs])
        fs = (ctypes.c_size_t * n)(*[h.size for h in hs])
        dp = (ctypes.c_void_p * n)(*frames_dev_ptrs)
        op = (ctypes.c_void_p * n)(*dst_dev_ptrs)
        cp = (ctypes.c_size_t * n)(*dst_capacities)
        self._keep = (hs, hp, fs, dp, op, cp)
        rep = self._lib.ozl_gpu_batch_plan(self._h, n, hp, fs, dp, op, cp)
        if rep.code:
            self._raise(rep)
        return rep.value

    def run(self, stream=0, graph=True):
        rep = self._lib.ozl_gpu_batch_run(self._h, stream, 1 if graph else 0)
        if rep.code:
            self._raise(rep)

    def check(self, stream=0):
        rep = self._lib.ozl_gpu_batch_check(self._h, stream)
        if rep.code:
            self._raise(rep)
        return rep.value

    def profile(self, stream=0, capacity=4096):
        """Per-launch (kind name, milliseconds, algorithmic bytes), run one by one."""
        ms = (ctypes.c_float * capacity)()
        kinds = (ctypes.c_int * capacity)()
        nb = (ctypes.c_uint64 * capacity)()
        rep = self._lib.ozl_gpu_batch_profile(self._h, stream, ms, kinds, nb, capacity)
        if rep.code:
            self._raise(rep)
        n = min(rep.value, capacity)
        return [(self._lib.ozl_gpu_kind_name(kinds[i]).decode(), ms[i], nb[i]) for i in range(n)]

    def run_host(self, h_in_ptr, in_bytes, h_out_ptr, out_bytes, stream=0, graph=True):
        """Host buffers in and out around one planned run (copies included)."""
        rep = self._lib.ozl_gpu_batch_run_host(self._h, h_in_ptr, in_bytes, h_out_ptr, out_bytes, stream,
                                               1 if graph else 0)
        if rep.code:
            self._raise(rep)
        return rep.value

    def launches(self):
        return self._lib.ozl_gpu_batch_launches(self._h)

    def sizes(self, n):
        p = self._lib.ozl_gpu_batch_sizes(self._h)
        return [p[i] for i in range(n)]


class GpuEncoder:
    """Batched compression on the device (frames identical to the reference's)."""

    def __init__(self):
        self._lib = library()
        self._h = self._lib.ozl_gpu_encoder_create()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ozl_gpu_encoder_free(h)
            self._h = None

    def bound(self, src_bytes):
        return self._lib.ozl_gpu_compress_bound(src_bytes)

    def compress_batch(self, src_ptrs, nb_elts, elt_widths, recipes, dst_ptrs, dst_caps, checksums=True, stream=0):
        """Device pointers in and out; returns the list of frame sizes."""
        n = len(src_ptrs)
        sp = (ctypes.c_void_p * n)(*src_ptrs)
        ne = (ctypes.c_size_t * n)(*nb_elts)
        ew = (ctypes.c_int * n)(*elt_widths)
        rc = (ctypes.c_int * n)(*recipes)
        dp = (ctypes.c_void_p * n)(*dst_ptrs)
        dc = (ctypes.c_size_t * n)(*dst_caps)
        fs = (ctypes.c_size_t * n)()
        rep = self._lib.ozl_gpu_compress_batch(self._h, n, sp, ne, ew, rc, dp, dc, fs, 1 if checksums else 0, stream)
        if rep.code:
            raise ZLError(rep.code, self._lib.ozl_gpu_encoder_error(self._h).decode())
        return [fs[i] for i in range(n)]
