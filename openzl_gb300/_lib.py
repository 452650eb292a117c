"""ctypes bindings of libopenzl_gb300 (names and semantics of include/openzl_gb300.h)."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libopenzl_gb300.so")
_lib = None


class ZLReport(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("value", ctypes.c_size_t)]


class NodeID(ctypes.Structure):
    _fields_ = [("nid", ctypes.c_uint)]


class GraphID(ctypes.Structure):
    _fields_ = [("gid", ctypes.c_uint)]


class OutputInfo(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("fixedWidth", ctypes.c_uint32), ("decompressedByteSize", ctypes.c_uint64),
                ("numElts", ctypes.c_uint64)]


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
        "ozl_frame_outputs": ([vp, sz, sz, vp, vp, vp, vp, vp, vp, vp], ZLReport),
        "ozl_frame_info": ([vp, sz, vp], ZLReport),
        "ozl_gpu_frame_info": ([vp, vp, sz, vp, vp], ZLReport),
        "ZL_TypedBuffer_rStringLens": ([vp], vp),
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
        "ozl_gpu_batch_timeline": ([vp, vp, vp, sz], ZLReport),
        "ozl_gpu_batch_host_timeline": ([vp, vp, sz, vp, sz, vp, vp, sz], ZLReport),
        "ozl_gpu_kind_name": ([ctypes.c_int], ctypes.c_char_p),
        "ozl_gpu_batch_run_host": ([vp, vp, sz, vp, sz, vp, ctypes.c_int], ZLReport),
        "ozl_gpu_batch_autotune": ([vp, vp, ctypes.c_int, vp, sz], ZLReport),
        "ozl_gpu_encoder_create": ([], vp),
        "ozl_gpu_encoder_free": ([vp], None),
        "ozl_gpu_compress_bound": ([sz], sz),
        "ozl_gpu_compress_batch": ([vp, sz, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, vp], ZLReport),
        "ozl_gpu_encoder_error": ([vp], ctypes.c_char_p),
        "ozl_gpu_encoder_phases": ([vp, vp, sz], ZLReport),
        "ozl_gpu_encoder_setParts": ([vp, ctypes.c_int], ZLReport),
        "ZL_DCtx_decompressTyped": ([vp, ctypes.POINTER(OutputInfo), vp, sz, vp, sz], ZLReport),
        "ZL_TypedBuffer_create": ([], vp),
        "ZL_TypedBuffer_free": ([vp], None),
        "ZL_TypedBuffer_createWrapSerial": ([vp, sz], vp),
        "ZL_TypedBuffer_createWrapStruct": ([vp, sz, sz], vp),
        "ZL_TypedBuffer_createWrapNumeric": ([vp, sz, sz], vp),
        "ZL_TypedBuffer_type": ([vp], ctypes.c_int),
        "ZL_TypedBuffer_byteSize": ([vp], sz),
        "ZL_TypedBuffer_rPtr": ([vp], vp),
        "ZL_TypedBuffer_numElts": ([vp], sz),
        "ZL_TypedBuffer_eltWidth": ([vp], sz),
        "ZL_DCtx_decompressTBuffer": ([vp, vp, vp, sz], ZLReport),
        "ZL_DCtx_decompressMultiTBuffer": ([vp, vp, sz, vp, sz], ZLReport),
        "ZL_FrameInfo_create": ([vp, sz], vp),
        "ZL_FrameInfo_free": ([vp], None),
        "ZL_FrameInfo_getFormatVersion": ([vp], ZLReport),
        "ZL_FrameInfo_getNumOutputs": ([vp], ZLReport),
        "ZL_FrameInfo_getOutputType": ([vp, ctypes.c_int], ZLReport),
        "ZL_FrameInfo_getDecompressedSize": ([vp, ctypes.c_int], ZLReport),
        "ZL_FrameInfo_getNumElts": ([vp, ctypes.c_int], ZLReport),
        "ZL_Compressor_create": ([], vp),
        "ZL_Compressor_free": ([vp], None),
        "ZL_Compressor_setParameter": ([vp, ctypes.c_int, ctypes.c_int], ZLReport),
        "ZL_Compressor_getParameter": ([vp, ctypes.c_int], ctypes.c_int),
        "ZL_Compressor_registerStaticGraph_fromNode1o": ([vp, NodeID, GraphID], GraphID),
        "ZL_Compressor_registerStaticGraph_fromPipelineNodes1o": ([vp, ctypes.POINTER(NodeID), sz, GraphID], GraphID),
        "ZL_Compressor_registerStaticGraph_fromNode": ([vp, NodeID, ctypes.POINTER(GraphID), sz], GraphID),
        "ZL_Compressor_registerTransposeSplitGraph": ([vp, GraphID], GraphID),
        "ZL_Compressor_registerTokenizeGraph": ([vp, ctypes.c_int, ctypes.c_bool, GraphID, GraphID], GraphID),
        "ZL_Compressor_selectStartingGraphID": ([vp, GraphID], ZLReport),
        "ZL_compressBound": ([sz], sz),
        "ZL_CCtx_create": ([], vp),
        "ZL_CCtx_free": ([vp], None),
        "ZL_CCtx_setParameter": ([vp, ctypes.c_int, ctypes.c_int], ZLReport),
        "ZL_CCtx_getParameter": ([vp, ctypes.c_int], ctypes.c_int),
        "ZL_CCtx_resetParameters": ([vp], ZLReport),
        "ZL_CCtx_refCompressor": ([vp, vp], ZLReport),
        "ZL_CCtx_compress": ([vp, vp, sz, vp, sz], ZLReport),
        "ZL_CCtx_getErrorContextString": ([vp, ZLReport], ctypes.c_char_p),
        "ZL_CCtx_compressTypedRef": ([vp, vp, sz, vp], ZLReport),
        "ZL_CCtx_compressMultiTypedRef": ([vp, vp, sz, vp, sz], ZLReport),
        "ZL_TypedRef_createSerial": ([vp, sz], vp),
        "ZL_TypedRef_createStruct": ([vp, sz, sz], vp),
        "ZL_TypedRef_createNumeric": ([vp, sz, sz], vp),
        "ZL_TypedRef_free": ([vp], None),
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


class FrameHeaderInfo(ctypes.Structure):
    """OZL_FrameInfo (include/openzl_gb300.h): a frame header's summary."""
    _fields_ = [("status", ctypes.c_int32), ("formatVersion", ctypes.c_uint32), ("nbOutputs", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("headerBytes", ctypes.c_uint64), ("output0Bytes", ctypes.c_uint64),
                ("extent", ctypes.c_uint64), ("output0Type", ctypes.c_int32), ("reserved", ctypes.c_uint32)]


def frame_header_info(frame):
    """ozl_frame_info: the header summary of a frame in host memory, parsed on
    the host (status 0 or the parse's ZL error code)."""
    f = _as_u8(frame)
    info = FrameHeaderInfo()
    _check(library().ozl_frame_info(f.ctypes.data if f.size else None, f.size, ctypes.byref(info)))
    return info


def frame_header_info_device(d_frame_ptrs, d_frame_sizes, n, d_info, stream=0):
    """ozl_gpu_frame_info: header summaries of n frames in device memory,
    parsed on the device. d_frame_ptrs / d_frame_sizes: device addresses of
    n 64-bit frame addresses / sizes; d_info: device address of n 48-byte
    records. Enqueued on `stream`."""
    return _check(library().ozl_gpu_frame_info(d_frame_ptrs, d_frame_sizes, n, d_info, stream))


def frame_outputs(frame):
    """ozl_frame_outputs: per output its offset in a batch destination, size
    in bytes (strings: content), ZL_Type value, element width, element count
    and (strings) the offset of the 4-byte lengths, as a list of dicts, and
    the destination bytes needed."""
    f = _as_u8(frame)
    n = _check(library().ozl_frame_outputs(f.ctypes.data, f.size, 0, None, None, None, None, None, None, None))
    offs = (ctypes.c_uint64 * max(n, 1))()
    sizes = (ctypes.c_uint64 * max(n, 1))()
    types = (ctypes.c_int * max(n, 1))()
    widths = (ctypes.c_uint32 * max(n, 1))()
    counts = (ctypes.c_uint64 * max(n, 1))()
    lens = (ctypes.c_uint64 * max(n, 1))()
    extent = ctypes.c_uint64()
    _check(library().ozl_frame_outputs(f.ctypes.data, f.size, n, offs, sizes, types, widths, counts, lens,
                                       ctypes.byref(extent)))
    return [{"offset": offs[o], "size": sizes[o], "type": types[o], "width": widths[o], "count": counts[o],
             "lens_offset": lens[o]} for o in range(n)], extent.value


# DParam values (include/openzl_gb300.h)
DPARAM_STICKY = 1
DPARAM_CHECK_COMPRESSED = 2
DPARAM_CHECK_CONTENT = 3
DPARAM_PARTS_PER_KIND = 1000  # OZL_DParam_partsPerKind
DPARAM_FSE_KERNEL = 1001  # OZL_DParam_fseKernel
DPARAM_CRITICAL_SYMBOLS = 1002  # OZL_DParam_criticalSymbols
DPARAM_SCHEDULE = 1003  # OZL_DParam_schedule
DPARAM_HOST_ROUNDS = 1004  # OZL_DParam_hostRounds
DPARAM_HOST_DEPTH = 1005  # OZL_DParam_hostDepth


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
        """ZL_DCtx_decompressTyped: host frame in, host bytes out (numpy uint8)."""
        data, _, _ = self.decompress_typed(frame, out)
        return data

    def decompress_typed(self, frame, out=None):
        """Returns (bytes as numpy uint8, ZL_Type value, element width)."""
        f = _as_u8(frame)
        n = get_decompressed_size(f)
        if out is None:
            out = np.empty(max(n, 1), np.uint8)
        info = OutputInfo()
        rep = self._lib.ZL_DCtx_decompressTyped(self._h, ctypes.byref(info), out.ctypes.data, out.nbytes,
                                                f.ctypes.data, f.size)
        if rep.code:
            raise ZLError(rep.code, self._err(rep))
        return out[: rep.value], info.type, info.fixedWidth

    def decompress_multi(self, frame, with_lengths=False):
        """ZL_DCtx_decompressMultiTBuffer: every output of the frame as
        [(bytes as numpy uint8, ZL_Type value, element width)], plus the
        string lengths (numpy uint32, None for other types) with
        `with_lengths`."""
        f = _as_u8(frame)
        fi = FrameInfo(f)
        n = fi.num_outputs()
        bufs = [self._lib.ZL_TypedBuffer_create() for _ in range(n)]
        try:
            arr = (ctypes.c_void_p * max(n, 1))(*bufs)
            rep = self._lib.ZL_DCtx_decompressMultiTBuffer(self._h, arr, n, f.ctypes.data, f.size)
            if rep.code:
                raise ZLError(rep.code, self._err(rep))
            res = []
            for b in bufs:
                size = self._lib.ZL_TypedBuffer_byteSize(b)
                ptr = self._lib.ZL_TypedBuffer_rPtr(b)
                data = np.ctypeslib.as_array((ctypes.c_uint8 * max(size, 1)).from_address(ptr))[:size].copy()
                t = self._lib.ZL_TypedBuffer_type(b)
                item = (data, t, self._lib.ZL_TypedBuffer_eltWidth(b))
                if with_lengths:
                    lens = None
                    if t == TYPE_STRING:
                        k = self._lib.ZL_TypedBuffer_numElts(b)
                        lp = self._lib.ZL_TypedBuffer_rStringLens(b)
                        lens = np.ctypeslib.as_array((ctypes.c_uint32 * max(k, 1)).from_address(lp))[:k].copy() if k else np.zeros(0, np.uint32)
                    item = item + (lens,)
                res.append(item)
            return res
        finally:
            for b in bufs:
                self._lib.ZL_TypedBuffer_free(b)

    def decompress_serial(self, frame, capacity):
        """ZL_DCtx_decompress (serial outputs only, as in the reference)."""
        f = _as_u8(frame)
        out = np.empty(max(capacity, 1), np.uint8)
        rep = self._lib.ZL_DCtx_decompress(self._h, out.ctypes.data, capacity, f.ctypes.data, f.size)
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

    def __init__(self, check_content=True, check_compressed=True, parts_per_kind=None, fse_kernel=None,
                 critical_symbols=None, schedule=None, host_rounds=None, host_depth=None):
        self._lib = library()
        self._h = self._lib.ozl_gpu_batch_create()
        if parts_per_kind is not None:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_PARTS_PER_KIND, int(parts_per_kind)))
        if fse_kernel is not None:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_FSE_KERNEL, int(fse_kernel)))
        if critical_symbols is not None:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_CRITICAL_SYMBOLS, int(critical_symbols)))
        if schedule is not None:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_SCHEDULE, int(schedule)))
        if host_rounds is not None:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_HOST_ROUNDS, int(host_rounds)))
        if host_depth is not None:
            _check(self._lib.ozl_gpu_batch_setParameter(self._h, DPARAM_HOST_DEPTH, int(host_depth)))
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

    def timeline(self, stream=0, capacity=4096):
        """One run with the branches in parallel and an event around every
        launch: (branch, kind name, level, ms its stream reached it, ms it
        ended), from the run's start."""
        rows = (ctypes.c_float * (5 * capacity))()
        rep = self._lib.ozl_gpu_batch_timeline(self._h, stream, rows, capacity)
        if rep.code:
            self._raise(rep)
        n = min(rep.value, capacity)
        return [(int(rows[5 * i]), self._lib.ozl_gpu_kind_name(int(rows[5 * i + 1])).decode(), int(rows[5 * i + 2]),
                 rows[5 * i + 3], rows[5 * i + 4]) for i in range(n)]

    def host_timeline(self, h_in_ptr, in_bytes, h_out_ptr, out_bytes, stream=0, capacity=64):
        """One host-buffer run with events: per round (ms in, ms decoded, ms
        out) from the run's start."""
        rows = (ctypes.c_float * (3 * capacity))()
        rep = self._lib.ozl_gpu_batch_host_timeline(self._h, h_in_ptr, in_bytes, h_out_ptr, out_bytes, stream,
                                                    rows, capacity)
        if rep.code:
            self._raise(rep)
        n = min(rep.value, capacity)
        return [(rows[3 * r], rows[3 * r + 1], rows[3 * r + 2]) for r in range(n)]

    def run_host(self, h_in_ptr, in_bytes, h_out_ptr, out_bytes, stream=0, graph=True):
        """Host buffers in and out around one planned run (copies included)."""
        rep = self._lib.ozl_gpu_batch_run_host(self._h, h_in_ptr, in_bytes, h_out_ptr, out_bytes, stream,
                                               1 if graph else 0)
        if rep.code:
            self._raise(rep)
        return rep.value

    def autotune(self, stream=0, reps=2, capacity=256):
        """Picks the launch shapes (chunks per CTA) by timing; returns the
        chosen shape per launch (0 = not tunable)."""
        shapes = (ctypes.c_uint32 * capacity)()
        rep = self._lib.ozl_gpu_batch_autotune(self._h, stream, reps, shapes, capacity)
        if rep.code:
            self._raise(rep)
        return list(shapes)[: min(rep.value, capacity)]

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

    def set_parts(self, parts):
        """Batches of 64 MiB or more run as `parts` (1..16) concurrent runs."""
        rep = self._lib.ozl_gpu_encoder_setParts(self._h, int(parts))
        if rep.code:
            raise ZLError(rep.code, "ozl_gpu_encoder_setParts failed")

    PHASES = ("front_end", "discovery", "histograms", "decisions", "bitstreams", "replay", "assembly")

    def phases(self):
        """Milliseconds of the last compress_batch's phases, by name."""
        ms = (ctypes.c_float * len(self.PHASES))()
        rep = self._lib.ozl_gpu_encoder_phases(self._h, ms, len(self.PHASES))
        if rep.code:
            raise ZLError(rep.code, "ozl_gpu_encoder_phases failed")
        return {k: round(ms[i], 3) for i, k in enumerate(self.PHASES)}


# ---------------------------------------------------------------------------
# Compression (ZL_Compressor / ZL_CCtx), mirroring the reference's C API.

NODE_DELTA_INT = 2
NODE_TRANSPOSE_SPLIT = 3
NODE_ZIGZAG = 4
NODE_BFLOAT16_DECONSTRUCT = 7
NODE_CONVERT_NUM_TO_TOKEN = 11
NODE_BITPACK_INT = 53
GRAPH_ILLEGAL = 0
GRAPH_STORE = 2
GRAPH_FSE = 3
GRAPH_HUFFMAN = 4
GRAPH_ENTROPY = 5
GRAPH_CONSTANT = 6
GRAPH_BITPACK = 8
GRAPH_FLATPACK = 9
CPARAM_STICKY = 1
CPARAM_FORMAT_VERSION = 4
CPARAM_COMPRESSED_CHECKSUM = 6
CPARAM_CONTENT_CHECKSUM = 7
TYPE_SERIAL, TYPE_STRUCT, TYPE_NUMERIC, TYPE_STRING = 1, 2, 4, 8


class Compressor:
    """ZL_Compressor: a graph registry (ids are plain ints here)."""

    def __init__(self):
        self._lib = library()
        self._h = self._lib.ZL_Compressor_create()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ZL_Compressor_free(h)
            self._h = None

    def set_parameter(self, p, v):
        _check(self._lib.ZL_Compressor_setParameter(self._h, p, v))

    def pipeline(self, nodes, dst):
        arr = (NodeID * len(nodes))(*[NodeID(n) for n in nodes])
        return self._lib.ZL_Compressor_registerStaticGraph_fromPipelineNodes1o(self._h, arr, len(nodes),
                                                                               GraphID(dst)).gid

    def node(self, node, dst):
        return self._lib.ZL_Compressor_registerStaticGraph_fromNode1o(self._h, NodeID(node), GraphID(dst)).gid

    def node_multi(self, node, dsts):
        arr = (GraphID * len(dsts))(*[GraphID(g) for g in dsts])
        return self._lib.ZL_Compressor_registerStaticGraph_fromNode(self._h, NodeID(node), arr, len(dsts)).gid

    def transpose_split(self, succ):
        return self._lib.ZL_Compressor_registerTransposeSplitGraph(self._h, GraphID(succ)).gid

    def tokenize(self, typ, sort, alphabet, indices):
        return self._lib.ZL_Compressor_registerTokenizeGraph(self._h, typ, sort, GraphID(alphabet),
                                                             GraphID(indices)).gid

    def select(self, gid):
        _check(self._lib.ZL_Compressor_selectStartingGraphID(self._h, GraphID(gid)))


class CCtx:
    """ZL_CCtx: compression context; compresses on the GPU."""

    def __init__(self):
        self._lib = library()
        self._h = self._lib.ZL_CCtx_create()
        self._comp = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ZL_CCtx_free(h)
            self._h = None

    def set_parameter(self, p, v):
        _check(self._lib.ZL_CCtx_setParameter(self._h, p, v))

    def ref_compressor(self, comp):
        self._comp = comp
        _check(self._lib.ZL_CCtx_refCompressor(self._h, comp._h))

    def _raise(self, rep):
        raise ZLError(rep.code, self._lib.ZL_CCtx_getErrorContextString(self._h, rep).decode())

    def compress(self, data, capacity=None):
        """ZL_CCtx_compress: serial input."""
        b = _as_u8(data)
        cap = capacity if capacity is not None else self._lib.ZL_compressBound(b.size)
        out = np.empty(max(cap, 1), np.uint8)
        rep = self._lib.ZL_CCtx_compress(self._h, out.ctypes.data, cap, b.ctypes.data if b.size else None, b.size)
        if rep.code:
            self._raise(rep)
        return out[: rep.value].copy()

    def compress_numeric(self, arr, capacity=None):
        """ZL_CCtx_compressTypedRef with a numeric ZL_TypedRef."""
        a = np.ascontiguousarray(arr)
        ref = self._lib.ZL_TypedRef_createNumeric(a.ctypes.data if a.size else None, a.itemsize, a.size)
        if not ref:
            raise ZLError(21, "ZL_TypedRef_createNumeric failed")
        cap = capacity if capacity is not None else self._lib.ZL_compressBound(a.nbytes)
        out = np.empty(max(cap, 1), np.uint8)
        try:
            rep = self._lib.ZL_CCtx_compressTypedRef(self._h, out.ctypes.data, cap, ref)
        finally:
            self._lib.ZL_TypedRef_free(ref)
        if rep.code:
            self._raise(rep)
        return out[: rep.value].copy()


class FrameInfo:
    """ZL_FrameInfo over a host frame (header only)."""

    def __init__(self, frame):
        self._lib = library()
        self._f = _as_u8(frame)
        self._h = self._lib.ZL_FrameInfo_create(self._f.ctypes.data, self._f.size)
        if not self._h:
            raise ZLError(12, "ZL_FrameInfo_create failed")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.ZL_FrameInfo_free(h)
            self._h = None

    def format_version(self):
        return _check(self._lib.ZL_FrameInfo_getFormatVersion(self._h))

    def num_outputs(self):
        return _check(self._lib.ZL_FrameInfo_getNumOutputs(self._h))

    def output_type(self, i=0):
        return _check(self._lib.ZL_FrameInfo_getOutputType(self._h, i))

    def decompressed_size(self, i=0):
        return _check(self._lib.ZL_FrameInfo_getDecompressedSize(self._h, i))

    def num_elts(self, i=0):
        return _check(self._lib.ZL_FrameInfo_getNumElts(self._h, i))


class Server:
    """Serving loop (ozl_server_*): continuous batching of decompress and
    compress requests with host buffers. Buffers are kept alive until their
    request has been polled."""

    def __init__(self, hbm_budget, workers=4, checksums=True):
        self._lib = library()
        L = self._lib
        if not getattr(L, "_server_sigs", False):
            vp, sz = ctypes.c_void_p, ctypes.c_size_t
            for name, args, res in [
                ("ozl_server_create", [sz, ctypes.c_int, ctypes.c_int], vp),
                ("ozl_server_free", [vp], None),
                ("ozl_server_submit_decompress", [vp, vp, sz, vp, sz], ctypes.c_uint64),
                ("ozl_server_submit_compress", [vp, vp, sz, ctypes.c_int, ctypes.c_int, vp, sz], ctypes.c_uint64),
                ("ozl_server_poll", [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ZLReport),
                                     ctypes.POINTER(ctypes.c_double), sz, ctypes.c_int], sz),
                ("ozl_server_in_flight", [vp], sz),
                ("ozl_server_stats", [vp, ctypes.POINTER(ctypes.c_double), sz], sz),
            ]:
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
            L._server_sigs = True
        self._h = L.ozl_server_create(hbm_budget, workers, 1 if checksums else 0)
        if not self._h:
            raise ZLError(70, "ozl_server_create failed")
        self._keep = {}

    def submit_decompress(self, frame, out):
        f = _as_u8(frame)
        i = self._lib.ozl_server_submit_decompress(self._h, f.ctypes.data, f.size, out.ctypes.data, out.nbytes)
        if not i:
            raise ZLError(21, "submit failed")
        self._keep[i] = (f, out)
        return i

    def submit_compress(self, arr, elt_width, recipe, out):
        a = np.ascontiguousarray(arr)
        if elt_width and a.nbytes % elt_width:
            raise ZLError(21, "input size is not a multiple of the element width")
        n = a.nbytes // elt_width if elt_width else a.nbytes
        i = self._lib.ozl_server_submit_compress(self._h, a.ctypes.data if a.size else None, n, elt_width, recipe,
                                                 out.ctypes.data, out.nbytes)
        if not i:
            raise ZLError(21, "submit failed")
        self._keep[i] = (a, out)
        return i

    _POLL = 4096

    def poll(self, wait_ms=0):
        """[(id, code, value, latency_us)] of completed requests."""
        if not hasattr(self, "_ids"):
            self._ids = (ctypes.c_uint64 * self._POLL)()
            self._res = (ZLReport * self._POLL)()
            self._lat = (ctypes.c_double * self._POLL)()
        ids, res, lat = self._ids, self._res, self._lat
        k = self._lib.ozl_server_poll(self._h, ids, res, lat, self._POLL, wait_ms)
        out = []
        for j in range(k):
            self._keep.pop(ids[j], None)
            out.append((ids[j], res[j].code, res[j].value, lat[j]))
        return out

    def in_flight(self):
        return self._lib.ozl_server_in_flight(self._h)

    STATS = ("decode_batches", "decode_requests", "decode_plan_s", "decode_run_s", "encode_batches",
             "encode_requests", "encode_s", "wait_s")

    def stats(self):
        """Cumulative worker statistics (ozl_server_stats), by name."""
        v = (ctypes.c_double * len(self.STATS))()
        k = self._lib.ozl_server_stats(self._h, v, len(self.STATS))
        return {name: round(v[i], 4) for i, name in enumerate(self.STATS[:k])}

    def close(self):
        if self._h:
            self._lib.ozl_server_free(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        self.close()
