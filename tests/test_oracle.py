"""CPU oracle: pinned against the reference's golden frames (and, where the
reference library is built in this container, against the reference itself)."""
import hashlib
import os

import numpy as np
import pytest

from conftest import ROOT, read_frame
from oracle import oracle

REF_DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver.so")


def test_oracle_decodes_every_golden_frame(manifest):
    assert len(manifest) >= 40
    for m in manifest:
        out, t, w = oracle.decompress(read_frame(m["case"]))
        assert hashlib.sha256(out.tobytes()).hexdigest() == m["sha256_in"], m["case"]


def test_oracle_detects_checksum_corruption(manifest):
    m = next(m for m in manifest if m["checksums"] and m["frame_bytes"] > 1000)
    fr = bytearray(read_frame(m["case"]))
    fr[len(fr) // 2] ^= 0x40
    with pytest.raises(ValueError):
        oracle.decompress(bytes(fr))


def test_oracle_older_format_versions(manifest):
    """Frames of format versions 8..20 (header-only differences, one block,
    checksums over the whole frame) decode, and a payload byte flipped in a
    v20 frame fails its compressed checksum, which spans the frame from its
    first byte."""
    old = [m for m in manifest if m.get("format_version", 23) < 21]
    assert {m["format_version"] for m in old} >= {8, 14, 15, 16, 20}
    for m in old:
        out, _, _ = oracle.decompress(read_frame(m["case"]))
        assert hashlib.sha256(out.tobytes()).hexdigest() == m["sha256_in"], m["case"]
    m = next(m for m in old if m["case"] == "v20_walk_u32_dz_tsplit_fse")
    fr = bytearray(read_frame(m["case"]))
    fr[len(fr) // 2] ^= 0x40
    with pytest.raises(ValueError):
        oracle.decompress(bytes(fr))


def test_oracle_decodes_multi_output_frames(manifest_multi):
    """Frames of several outputs (output o in stream slot total-1-o of each
    block, the content checksum over the block's outputs one after another)."""
    assert any(len(m["outputs"]) > 14 for m in manifest_multi)  # extended output count
    assert any(o["type"] == 8 for m in manifest_multi for o in m["outputs"])  # string outputs
    for m in manifest_multi:
        outs = oracle.decompress_multi(read_frame(m["case"]), with_lengths=True)
        assert len(outs) == len(m["outputs"]), m["case"]
        for (data, t, w, lens), o in zip(outs, m["outputs"]):
            assert hashlib.sha256(data.tobytes()).hexdigest() == o["sha256"], m["case"]
            assert t == o["type"] and w == (o["elt_width"] or 1), m["case"]
            if t == 8:
                assert hashlib.sha256(lens.astype("<u4").tobytes()).hexdigest() == o["sha256_lens"], m["case"]
    m = next(m for m in manifest_multi if m["case"] == "multi3_ts_delta_flatpack")
    fr = bytearray(read_frame(m["case"]))
    fr[len(fr) // 2] ^= 0x40
    with pytest.raises(ValueError):
        oracle.decompress_multi(bytes(fr))


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_oracle_matches_reference_on_string_frames():
    """String inputs (separate_string_components, then content and lengths
    through store, FSE or Huffman graphs) at format versions 15 to 23: the
    oracle gives back the content and the lengths; wrong lengths are
    corruption."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    f = ref.ref_compress_string
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                  ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(17)
    words = [bytes(rng.integers(97, 123, int(rng.integers(0, 9))).astype(np.uint8)) for _ in range(100)]
    for nstr in (1, 7, 3000):
        strs = [words[i] for i in (rng.zipf(1.2, nstr) - 1) % len(words)]
        content = np.frombuffer(b"".join(strs), np.uint8).copy()
        lens = np.array([len(x) for x in strs], np.uint32)
        for recipe in (100, 101, 102):
            for v in (15, 20, 21, 23):
                for cs in (0, 1):
                    dst = np.zeros(content.size * 2 + lens.nbytes * 2 + 65536, np.uint8)
                    r = f(recipe, content.ctypes.data if content.size else None, content.size, lens.ctypes.data,
                          lens.size, dst.ctypes.data, dst.size, cs, v)
                    assert r > 0, (recipe, v, nstr)
                    (data, t, w, got), = oracle.decompress_multi(dst[:r].tobytes(), with_lengths=True)
                    assert t == 8 and data.tobytes() == content.tobytes() and np.array_equal(got, lens), (recipe, v)


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_oracle_matches_reference_on_multi_input_frames():
    """Seeded multi-input frames (1 to 40 inputs, mixed recipes, format
    versions 15 to 23, with and without checksums) decode in the oracle."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    f = ref.ref_compress_multi
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(9)

    def spec():
        k = int(rng.integers(0, 6))
        n = int(rng.choice([1, 5, 300, 5000, 40000]))
        walk = (1000 + np.cumsum(rng.integers(-50, 51, n)))
        return [(1, walk.astype(np.uint32), 4), (2, (1000 + np.cumsum(rng.integers(0, 900, n))).astype(np.uint64), 8),
                (8, (rng.zipf(1.3, n) % 256).astype(np.uint8), 0), (7, (rng.zipf(1.3, n) % 40).astype(np.uint8), 0),
                (9, walk.astype(np.uint16), 2), (0, rng.integers(0, 256, n).astype(np.uint8), 0)][k]

    for trial in range(30):
        nb = int(rng.choice([1, 2, 3, 5, 14, 15, 16, 20, 40]))
        specs = [spec() for _ in range(nb)]
        v = int(rng.choice([15, 16, 20, 21, 22, 23]))
        cs = int(rng.integers(0, 2))
        arrs = [np.ascontiguousarray(a) for _, a, _ in specs]
        cap = sum(a.nbytes for a in arrs) * 2 + 8192 * nb
        dst = np.zeros(cap, np.uint8)
        r = f(nb, (ctypes.c_int * nb)(*[s[0] for s in specs]), (ctypes.c_void_p * nb)(*[a.ctypes.data for a in arrs]),
              (ctypes.c_size_t * nb)(*[a.size if w else a.nbytes for (_, _, w), a in zip(specs, arrs)]),
              (ctypes.c_int * nb)(*[s[2] for s in specs]), dst.ctypes.data, cap, cs, v)
        assert r > 0, (trial, r)
        outs = oracle.decompress_multi(dst[:r].tobytes())
        assert [o.tobytes() for o, _, _ in outs] == [a.tobytes() for a in arrs], (trial, nb, v, cs)


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_oracle_matches_reference_at_older_format_versions():
    """Seeded inputs compressed by the reference at every format version from
    15 to 20 (and 14 for graphs without entropy coding) decode in the oracle."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(7)
    cases = [(1, 4, np.uint32), (2, 8, np.int64), (3, 2, np.uint16), (4, 1, np.uint8), (9, 4, np.uint32),
             (10, 8, np.uint64), (11, 2, np.uint16), (12, 4, np.uint32)]
    for v in range(14, 21):
        for recipe, w, dt in cases:
            if v == 14 and recipe < 9:
                continue  # entropy coding before v15 uses the deprecated codecs
            for n in (1, 1000, 40001):
                arr = (500 + np.cumsum(rng.integers(-50, 51, n))).astype(dt)
                cap = arr.nbytes * 2 + 4096
                dst = np.zeros(cap, np.uint8)
                for cs in (0, 1):
                    r = ref.ref_compress(recipe, arr.ctypes.data, n, w, dst.ctypes.data, cap, cs, v)
                    assert r > 0, (v, recipe, n)
                    out, _, _ = oracle.decompress(dst[:r].tobytes())
                    assert out.tobytes() == arr.tobytes(), (v, recipe, n, cs)


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_oracle_matches_reference_on_2byte_entropy_graphs():
    """2-byte numbers through the Huffman and entropy graphs (the 16-bit
    branch of the entropy chunk: constant, bit packing, store, tokenize or
    huffman_struct_v2, chunked from 100000 elements): the oracle's frames
    equal the reference's."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(3)
    for recipe in (8, 17):
        for n in (2, 3, 100, 999, 1001, 5000, 40000, 99999, 100000, 140000):
            for a in ((rng.zipf(1.3, n) % 3000).astype(np.uint16), (rng.zipf(1.2, n) % 200).astype(np.uint16),
                      np.minimum(rng.geometric(1 / 3000, n), 65535).astype(np.uint16),
                      rng.integers(0, 65536, n).astype(np.uint16), rng.integers(0, 40, n).astype(np.uint16),
                      np.full(n, 77, np.uint16), rng.choice(np.array([5, 60000], np.uint16), n)):
                dst = np.zeros(4 * n + 4096, np.uint8)
                r = ref.ref_compress(recipe, a.ctypes.data, n, 2, dst.ctypes.data, dst.size, 1, 0)
                assert r > 0
                assert oracle.compress(recipe, a, 2).tobytes() == dst[:r].tobytes(), (recipe, n)


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_xxh3_every_length_class_matches_reference():
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_xxh3_64.restype = ctypes.c_uint64
    ref.ref_xxh3_64.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    rng = np.random.default_rng(1)
    for n in [0, 1, 3, 4, 8, 9, 16, 17, 100, 128, 129, 240, 241, 1024, 1025, 1088, 5000, 100000]:
        b = rng.integers(0, 256, n).astype(np.uint8)
        assert oracle.xxh3_64(b.tobytes()) == ref.ref_xxh3_64(b.ctypes.data, n), n


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_oracle_matches_reference_on_seeded_inputs():
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(99)
    for recipe, w, dt in [(1, 4, np.uint32), (2, 8, np.int64), (3, 2, np.uint16), (4, 8, np.uint64),
                          (3, 1, np.uint8), (4, 4, np.uint32)]:
        for n in (1, 2, 999, 1000, 33000, 150001):
            arr = (500 + np.cumsum(rng.integers(-50, 51, n))).astype(dt)
            cap = arr.nbytes * 2 + 4096
            dst = np.zeros(cap, np.uint8)
            r = ref.ref_compress(recipe, arr.ctypes.data, n, w, dst.ctypes.data, cap, 1, 0)
            assert r > 0
            out, _, _ = oracle.decompress(dst[:r].tobytes())
            assert out.tobytes() == arr.tobytes(), (recipe, w, n)


def test_oracle_encoder_reproduces_every_golden_frame(manifest):
    """The CPU encoder restatement emits the reference's exact frame bytes."""
    for m in manifest:
        if m.get("decode_only"):
            continue
        fr = read_frame(m["case"])
        data, _, w = oracle.decompress(fr)
        width = m["elt_width"]
        arr = data.view({0: np.uint8, 1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[width])
        got = oracle.compress(m["recipe"], arr, width, checksums=bool(m["checksums"]))
        assert hashlib.sha256(got.tobytes()).hexdigest() == m["sha256_frame"], m["case"]


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference library not built here")
def test_oracle_encoder_matches_reference_on_seeded_inputs():
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(1234)
    cases = []
    for w, dt in [(1, np.uint8), (2, np.uint16), (4, np.uint32), (8, np.uint64)]:
        for recipe in (1, 2, 3, 4, 9, 10, 11, 12):
            for n in (1, 9, 999, 40000, 120000):
                cases.append((recipe, (7000 + np.cumsum(rng.integers(-3000, 3001, n))).astype(dt), w))
    for recipe in (7, 8):
        for n in (2, 10, 1001, 100000, 140000):
            for k in (2, 5, 256):
                cases.append((recipe, (rng.zipf(1.2, n) % k).astype(np.uint8), 0))
    keys = rng.integers(-2**31, 2**31, 1000).astype(np.int32)
    cases.append((5, keys[(rng.zipf(1.1, 50000) - 1) % 1000], 4))
    cases.append((16, keys[(rng.zipf(1.1, 50000) - 1) % 300], 4))
    bf = rng.normal(0, 0.02, 70000).astype(np.float32).view(np.uint32)
    cases.append((6, (bf >> 16).astype(np.uint16), 2))
    for recipe, arr, w in cases:
        for cs in (1, 0):
            cap = arr.nbytes * 2 + 65536
            dst = np.zeros(cap, np.uint8)
            n = arr.size if w else arr.nbytes
            r = ref.ref_compress(recipe, arr.ctypes.data, n, w, dst.ctypes.data, cap, cs, 0)
            assert r > 0
            got = oracle.compress(recipe, arr, w, checksums=bool(cs))
            assert got.tobytes() == dst[:r].tobytes(), (recipe, w, arr.size, cs)


def equal_count_cases(n=80):
    """Serial inputs whose byte histograms (one chunk) hold 9 to 29 symbols
    of count 164, beside up to five large counts and 20 to 150 counts of 60
    to 239. The reference's Huffman sort quicksorts its rank buckets from the
    count-164 bucket on (its distinct-count cutoff is 165): that reorders
    these equal counts and decides which of them get the longer codes. Frames
    of about one case in six differ when the bucket is left in symbol order."""
    rng = np.random.default_rng(1640)
    out = []
    for _ in range(n):
        counts = {s: int(rng.integers(2000, 9000)) for s in range(int(rng.integers(1, 6)))}
        syms = rng.permutation(np.arange(len(counts), 256))
        k = int(rng.integers(9, 30))
        for s in syms[:k]:
            counts[int(s)] = 164
        for s in syms[k:k + int(rng.integers(20, 150))]:
            counts[int(s)] = int(rng.integers(60, 240))
        arr = np.concatenate([np.full(c, s, np.uint8) for s, c in counts.items()])
        rng.shuffle(arr)
        out.append(arr)
    return out


def test_oracle_matches_reference_on_equal_count_histograms():
    """Frames through the Huffman and entropy graphs equal the reference's
    when a group of equal counts sits in the Huffman sort's count-164 bucket."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    bad = []
    for k, arr in enumerate(equal_count_cases()):
        for recipe in (8, 17):
            cap = arr.nbytes * 2 + 65536
            dst = np.zeros(cap, np.uint8)
            r = ref.ref_compress(recipe, arr.ctypes.data, arr.nbytes, 0, dst.ctypes.data, cap, 1, 0)
            assert r > 0
            if oracle.compress(recipe, arr, 0).tobytes() != dst[:r].tobytes():
                bad.append((k, recipe))
    assert not bad, bad


def constant_graph_cases():
    """Constant numbers of 1, 2, 4 and 8 bytes (and serial bytes) through
    the constant graph, from 10 to 300,000 elements."""
    out = []
    for w, dt in [(1, np.uint8), (2, np.uint16), (4, np.uint32), (8, np.uint64)]:
        for n in (10, 255, 1000, 100001, 300000):
            out.append((np.full(n, 0x0102030405060708 % (256 ** w), dt), w))
    out.append((np.full(5000, 9, np.uint8), 0))
    return out


def test_oracle_constant_graph_matches_reference():
    """Numbers reach the constant graph through a conversion to struct, as
    in the reference (the graph takes serial or struct input); frames are
    equal, and input that is not constant fails in both."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    for arr, w in constant_graph_cases():
        cap = arr.nbytes * 2 + 65536
        dst = np.zeros(cap, np.uint8)
        r = ref.ref_compress(13, arr.ctypes.data, arr.size if w else arr.nbytes, w, dst.ctypes.data, cap, 1, 0)
        assert r > 0
        assert oracle.compress(13, arr, w).tobytes() == dst[:r].tobytes(), (w, arr.size)
    for w, dt in [(0, np.uint8), (1, np.uint8), (4, np.uint32)]:
        arr = np.full(1000, 7, dt)
        arr[500] = 8
        dst = np.zeros(8192, np.uint8)
        assert ref.ref_compress(13, arr.ctypes.data, arr.size if w else arr.nbytes, w, dst.ctypes.data, 8192, 1, 0) < 0
        with pytest.raises(Exception):
            oracle.compress(13, arr, w)


def test_oracle_matches_reference_on_random_recipes():
    """A seeded random sweep: every numeric recipe, widths 1-8, six data
    shapes (uniform, random walks, Zipf, constant, geometric, runs), sizes
    around the 32 KiB and 100,000-element chunking boundaries; where the
    reference compresses, the frames are equal and the reference's frame
    decodes to the input in the oracle."""
    import ctypes

    ref = ctypes.CDLL(REF_DRIVER)
    ref.ref_compress.restype = ctypes.c_int64
    ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(2809)
    sizes = [1, 2, 3, 5, 17, 255, 999, 1000, 1001, 4096, 32767, 32768, 32769, 65536, 99999, 100000, 100001, 131072]
    dts = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}

    def data(shape, n, w):
        dt = dts[w]
        if shape == 0:
            return rng.integers(0, 256 ** min(w, 4), n, dtype=np.uint64).astype(dt)
        if shape == 1:
            s = int(rng.integers(1, 70000))
            return (7000 + np.cumsum(rng.integers(-s, s, n))).astype(dt)
        if shape == 2:
            return (rng.zipf(1.0 + rng.random() * 1.5, n) % int(rng.integers(2, 70000))).astype(dt)
        if shape == 3:
            return np.full(n, int(rng.integers(0, 255)), dt)
        if shape == 4:
            return rng.geometric(1 / float(rng.integers(2, 5000)), n).astype(dt)
        return np.repeat(rng.integers(0, 1000, n // 7 + 1), 7)[:n].astype(dt)

    checked, bad = 0, []
    for k in range(1500):
        recipe = int(rng.choice([1, 2, 3, 4, 9, 10, 11, 12, 13, 15, 17, 7, 8, 14, 5, 16]))
        n = int(rng.choice(sizes))
        shape = int(rng.integers(0, 6))
        if recipe in (7, 8, 14):
            w, arr = 0, data(shape, n, 1)
        elif recipe in (5, 16):
            w, arr = 4, (data(shape, n, 4) % int(rng.integers(2, 3000))).astype(np.uint32)
        else:
            w = int(rng.choice([1, 2, 4, 8]))
            arr = data(shape, n, w)
        cap = arr.nbytes * 2 + 65536
        dst = np.zeros(cap, np.uint8)
        r = ref.ref_compress(recipe, arr.ctypes.data, arr.size if w else arr.nbytes, w, dst.ctypes.data, cap, 1, 0)
        if r <= 0:
            continue
        checked += 1
        if oracle.compress(recipe, arr, w).tobytes() != dst[:r].tobytes():
            bad.append((k, recipe, w, n, shape))
        # the reference's frame decodes to the input in the oracle
        if oracle.decompress(dst[:r].copy())[0].tobytes() != arr.tobytes():
            bad.append((k, recipe, w, n, shape, "decode"))
    assert checked > 1300 and not bad, (checked, bad[:10])


def tablelog12_cases():
    """Frames whose FSE chunks use table log 12, the decoders' limit (the
    reference's encoder stops at 11): 99,999-symbol unchunked streams, a
    chunked stream and transpose-split planes."""
    rng = np.random.default_rng(1212)
    cases = [(7, (rng.zipf(1.1, 99999) % 256).astype(np.uint8), 0),
             (7, (rng.zipf(1.05, 99999) % 256).astype(np.uint8), 0),
             (7, (rng.zipf(1.1, 250000) % 256).astype(np.uint8), 0),
             (3, (1000 + np.cumsum(rng.integers(-40000, 40001, 99999))).astype(np.uint16), 2)]
    return [(r, a, w, oracle.compress_tablelog12(r, a, w)) for r, a, w in cases]


def test_tablelog12_frames_decode_in_oracle_and_reference():
    import ctypes

    cases = tablelog12_cases()
    ref = None
    if os.path.exists(REF_DRIVER):
        ref = ctypes.CDLL(REF_DRIVER)
        ref.ref_decompress_into.restype = ctypes.c_int64
        ref.ref_decompress_into.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                            ctypes.c_int]
    for recipe, arr, w, fr in cases:
        # the frame differs from the table-log-11 frame the reference would write
        assert fr.tobytes() != oracle.compress(recipe, arr, w).tobytes()
        data, _, _ = oracle.decompress(fr)
        assert data.tobytes() == arr.tobytes()
        if ref is not None:
            out = np.zeros(arr.nbytes + 64, np.uint8)
            n = ref.ref_decompress_into(fr.ctypes.data, fr.size, out.ctypes.data, out.size, 1)
            assert n == arr.nbytes and out[:n].tobytes() == arr.tobytes()


def huf_tablelog12_cases():
    """Frames whose Huffman chunks use table log 12, the decoders' limit (the
    reference's encoder stops at 11): skewed bytes whose rarest codes reach
    12 bits, unchunked and in 32 KiB chunks, and a bit-packed numeric graph."""
    rng = np.random.default_rng(1213)
    geo = lambda p, n: np.minimum(rng.geometric(p, n) - 1, 255)  # noqa: E731
    cases = [(8, geo(0.2, 90000).astype(np.uint8), 0),
             (8, geo(0.15, 400000).astype(np.uint8), 0),
             (4, np.cumsum(geo(0.3, 60000)).astype(np.uint32), 4),
             (4, np.cumsum(geo(0.25, 60000) + 1).astype(np.uint16), 2)]
    return [(r, a, w, oracle.compress_huf_tablelog12(r, a, w)) for r, a, w in cases]


def test_huf_tablelog12_frames_decode_in_oracle_and_reference():
    import ctypes

    cases = huf_tablelog12_cases()
    ref = None
    if os.path.exists(REF_DRIVER):
        ref = ctypes.CDLL(REF_DRIVER)
        ref.ref_decompress_into.restype = ctypes.c_int64
        ref.ref_decompress_into.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                            ctypes.c_int]
    for recipe, arr, w, fr in cases:
        assert fr.tobytes() != oracle.compress(recipe, arr, w).tobytes()
        data, _, _ = oracle.decompress(fr)
        assert data.tobytes() == arr.tobytes()
        if ref is not None:
            out = np.zeros(arr.nbytes + 64, np.uint8)
            n = ref.ref_decompress_into(fr.ctypes.data, fr.size, out.ctypes.data, out.size, 1)
            assert n == arr.nbytes and out[:n].tobytes() == arr.tobytes()


def test_oracle_frames_of_many_chunks():
    """A concatenation of more than 300 entropy chunks (a 12 MB serial input
    cut into 32 KiB chunks) decodes, and the encoder's frame equals the
    reference's."""
    import ctypes

    rng = np.random.default_rng(300)
    a = (rng.zipf(1.3, 12 << 20) % 256).astype(np.uint8)
    fr = oracle.compress(8, a, 0)
    data, _, _ = oracle.decompress(fr)
    assert data.tobytes() == a.tobytes()
    if os.path.exists(REF_DRIVER):
        ref = ctypes.CDLL(REF_DRIVER)
        ref.ref_compress.restype = ctypes.c_int64
        ref.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
        dst = np.zeros(a.size * 2 + 65536, np.uint8)
        n = ref.ref_compress(8, a.ctypes.data, a.size, 0, dst.ctypes.data, dst.size, 1, 0)
        assert n == fr.size and dst[:n].tobytes() == fr.tobytes()
