"""Compression through the reference's API (ZL_Compressor graphs, ZL_CCtx)
on the GPU: every graph built the way a reference user builds it produces
the reference's frame (pinned through the oracle), and typed decompression
and typed buffers behave as the reference's do."""
import ctypes

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _graph(oz, comp, recipe):
    a = oz.api
    if recipe == 0:
        return a.GRAPH_STORE
    if recipe == 1:
        return comp.pipeline([a.NODE_DELTA_INT, a.NODE_ZIGZAG, a.NODE_CONVERT_NUM_TO_TOKEN],
                             comp.transpose_split(a.GRAPH_FSE))
    if recipe == 2:
        return comp.pipeline([a.NODE_DELTA_INT, a.NODE_ZIGZAG], comp.node(a.NODE_BITPACK_INT, a.GRAPH_HUFFMAN))
    if recipe == 3:
        return comp.pipeline([a.NODE_DELTA_INT, a.NODE_CONVERT_NUM_TO_TOKEN], comp.transpose_split(a.GRAPH_FSE))
    if recipe == 4:
        return comp.node(a.NODE_DELTA_INT, comp.node(a.NODE_BITPACK_INT, a.GRAPH_HUFFMAN))
    if recipe == 7:
        return a.GRAPH_FSE
    if recipe == 8:
        return a.GRAPH_HUFFMAN
    if recipe == 9:
        return comp.node(a.NODE_DELTA_INT, a.GRAPH_STORE)
    if recipe == 10:
        return comp.node(a.NODE_ZIGZAG, a.GRAPH_STORE)
    if recipe == 11:
        return comp.node(a.NODE_BITPACK_INT, a.GRAPH_STORE)
    if recipe == 12:
        return comp.node(a.NODE_CONVERT_NUM_TO_TOKEN, comp.transpose_split(a.GRAPH_STORE))
    if recipe == 13:
        return a.GRAPH_CONSTANT
    if recipe == 14:
        return a.GRAPH_FLATPACK
    if recipe == 15:
        return a.GRAPH_BITPACK
    if recipe == 17:
        return a.GRAPH_ENTROPY
    if recipe in (5, 16):
        return comp.tokenize(a.TYPE_NUMERIC, recipe == 16, a.GRAPH_STORE, comp.node(a.NODE_BITPACK_INT, a.GRAPH_HUFFMAN))
    if recipe == 6:
        return comp.node_multi(a.NODE_BFLOAT16_DECONSTRUCT, [a.GRAPH_STORE, a.GRAPH_FSE])
    raise ValueError(recipe)


def _cases():
    rng = np.random.default_rng(31)
    c = []
    for recipe in (1, 2, 3, 4, 9, 10, 11, 12):
        for dt in (np.uint8, np.uint16, np.uint32, np.uint64):
            for n in (5, 3000, 150000):
                a = (1000 + np.cumsum(rng.integers(-700, 701, n))).astype(dt)
                c.append((recipe, a))
    keys = rng.integers(0, 2**31, 10000).astype(np.uint32)
    for n in (50, 40000):
        c.append((5, keys[(rng.zipf(1.1, n) - 1) % keys.size]))
        c.append((16, keys[(rng.zipf(1.1, n) - 1) % keys.size]))
    c.append((6, (rng.normal(0, 0.02, 30000).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)))
    for recipe in (0, 7, 8, 13, 14, 15):
        for n in (3, 5000, 120000):
            a = (rng.zipf(1.3, n) % 41).astype(np.uint8)
            if recipe == 13:
                a[:] = 7
            c.append((recipe, a))
    # the entropy graph: Huffman, FSE (low entropy), flatpack and store chunks
    for n in (3, 5000, 120000, 260000):
        c.append((17, (rng.zipf(1.3, n) % 41).astype(np.uint8)))
        c.append((17, np.where(rng.random(n) < 0.98, 0, rng.integers(1, 256, n)).astype(np.uint8)))
    c.append((17, rng.integers(0, 256, 40000).astype(np.uint8)))
    return c


@pytest.mark.parametrize("checksums", [True, False])
def test_cctx_frames_equal_reference_frames(gpu_lib, checksums):
    import openzl_gb300 as oz

    a = oz.api
    bad = []
    for recipe, arr in _cases():
        comp = oz.Compressor()
        comp.select(_graph(oz, comp, recipe))
        cctx = oz.CCtx()
        cctx.ref_compressor(comp)
        cctx.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
        if not checksums:
            cctx.set_parameter(a.CPARAM_CONTENT_CHECKSUM, 2)
            cctx.set_parameter(a.CPARAM_COMPRESSED_CHECKSUM, 2)
        serial = recipe in (0, 7, 8, 13, 14, 15, 17)
        got = cctx.compress(arr.tobytes()) if serial else cctx.compress_numeric(arr)
        want = oracle.compress(recipe, arr, 0 if serial else arr.itemsize, checksums=checksums)
        if got.tobytes() != want.tobytes():
            bad.append((recipe, arr.dtype.name, arr.size, got.size, want.size))
        # round trip with typed decompression
        d = oz.DCtx()
        data, typ, width = d.decompress_typed(got)
        assert data.tobytes() == arr.tobytes(), (recipe, arr.dtype.name, arr.size)
        assert typ == (a.TYPE_SERIAL if serial else a.TYPE_NUMERIC)
        assert width == (1 if serial else arr.itemsize)
    assert not bad, bad[:10]


def test_cctx_2byte_numbers_through_huffman_and_entropy_graphs(gpu_lib):
    """ZL_GRAPH_HUFFMAN and ZL_GRAPH_ENTROPY on 2-byte numeric input: the
    16-bit chunk path (tokenize, bit packing, store, constant or
    huffman_struct_v2) gives the reference's frames, and they decode back to
    typed numeric output."""
    import openzl_gb300 as oz

    a = oz.api
    rng = np.random.default_rng(41)
    arrs = []
    for n in (3, 1001, 50000, 150000):
        arrs.append((rng.zipf(1.3, n) % 3000).astype(np.uint16))
        arrs.append((rng.zipf(1.2, n) % 150).astype(np.uint16))
        arrs.append(rng.integers(0, 30, n).astype(np.uint16))
    arrs.append(np.full(4000, 1234, np.uint16))
    arrs.append(rng.integers(0, 65536, 9000).astype(np.uint16))
    bad = []
    for recipe in (8, 17):
        for arr in arrs:
            comp = oz.Compressor()
            comp.select(_graph(oz, comp, recipe))
            cctx = oz.CCtx()
            cctx.ref_compressor(comp)
            cctx.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
            got = cctx.compress_numeric(arr)
            want = oracle.compress(recipe, arr, 2)
            if got.tobytes() != want.tobytes():
                bad.append((recipe, arr.size, got.size, want.size))
            data, typ, width = oz.DCtx().decompress_typed(got)
            assert data.tobytes() == arr.tobytes() and typ == a.TYPE_NUMERIC and width == 2, (recipe, arr.size)
    assert not bad, bad


def test_decompress_rejects_typed_outputs_like_the_reference(gpu_lib):
    import openzl_gb300 as oz

    a = oz.api
    arr = np.arange(5000, dtype=np.uint32)
    comp = oz.Compressor()
    comp.select(comp.node(a.NODE_DELTA_INT, a.GRAPH_STORE))
    cctx = oz.CCtx()
    cctx.ref_compressor(comp)
    cctx.set_parameter(a.CPARAM_STICKY, 1)
    cctx.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
    frame = cctx.compress_numeric(arr)
    d = oz.DCtx()
    with pytest.raises(oz.ZLError) as e:  # decompress2.c:1850-1856
        d.decompress_serial(frame, arr.nbytes)
    assert e.value.code == 1
    # sticky parameters: the same CCtx compresses again without re-setting them
    assert cctx.compress_numeric(arr).tobytes() == frame.tobytes()
    # a serial frame goes through ZL_DCtx_decompress
    comp2 = oz.Compressor()
    comp2.select(a.GRAPH_HUFFMAN)
    c2 = oz.CCtx()
    c2.ref_compressor(comp2)
    c2.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
    raw = (np.arange(20000) % 13).astype(np.uint8).tobytes()
    f2 = c2.compress(raw)
    assert d.decompress_serial(f2, len(raw)).tobytes() == raw
    with pytest.raises(oz.ZLError) as e:
        d.decompress_serial(f2, len(raw) - 1)
    assert e.value.code == 5
    # compressed output larger than the capacity
    c2.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
    with pytest.raises(oz.ZLError) as e:
        c2.compress(raw, capacity=8)
    assert e.value.code == 5


def test_typed_buffers(gpu_lib):
    import openzl_gb300 as oz

    lib = oz.library()
    arr = (np.arange(40000) * 7).astype(np.uint16)
    frame = oracle.compress(3, arr, 2)
    f = np.frombuffer(frame.tobytes(), np.uint8)
    d = oz.DCtx()
    # DCtx-owned buffer
    tb = lib.ZL_TypedBuffer_create()
    r = lib.ZL_DCtx_decompressTBuffer(d._h, tb, f.ctypes.data, f.size)
    assert r.code == 0 and r.value == arr.nbytes
    assert lib.ZL_TypedBuffer_type(tb) == 4 and lib.ZL_TypedBuffer_eltWidth(tb) == 2
    assert lib.ZL_TypedBuffer_numElts(tb) == arr.size
    got = ctypes.string_at(lib.ZL_TypedBuffer_rPtr(tb), lib.ZL_TypedBuffer_byteSize(tb))
    assert got == arr.tobytes()
    lib.ZL_TypedBuffer_free(tb)
    # wrapped numeric buffer of the right width, then of the wrong width
    out = np.zeros(arr.size, np.uint16)
    tb = lib.ZL_TypedBuffer_createWrapNumeric(out.ctypes.data, 2, out.size)
    r = lib.ZL_DCtx_decompressTBuffer(d._h, tb, f.ctypes.data, f.size)
    assert r.code == 0 and np.array_equal(out, arr)
    lib.ZL_TypedBuffer_free(tb)
    out4 = np.zeros(arr.size, np.uint32)
    tb = lib.ZL_TypedBuffer_createWrapNumeric(out4.ctypes.data, 4, out4.size)
    r = lib.ZL_DCtx_decompressTBuffer(d._h, tb, f.ctypes.data, f.size)
    assert r.code != 0
    lib.ZL_TypedBuffer_free(tb)
    # multi-output entry point with one output: returns the number of
    # buffers filled (zl_decompress.h:511-526)
    tb = lib.ZL_TypedBuffer_create()
    arrp = (ctypes.c_void_p * 1)(tb)
    r = lib.ZL_DCtx_decompressMultiTBuffer(d._h, arrp, 1, f.ctypes.data, f.size)
    assert r.code == 0 and r.value == 1
    assert lib.ZL_TypedBuffer_byteSize(tb) == arr.nbytes and lib.ZL_TypedBuffer_eltWidth(tb) == 2
    lib.ZL_TypedBuffer_free(tb)
