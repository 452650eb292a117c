"""Generates the golden frames under tests/golden/ with the reference library.

Run in a container that holds the reference sources (it builds
oracle/_ref/ with oracle/ref.mk first). Each case is the frame the reference
compressor produced for a seeded input, plus a manifest entry holding the
SHA-256 of that input. The tests decode the frames with the GPU library and
with the CPU oracle and check both against the recorded input hash; the
encoders re-create every frame not marked decode_only.

    python tests/golden/make_golden.py
"""
import ctypes
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# recipe numbers follow oracle/ref_driver.c
CASES = []


def walk(rng, n, dtype, step, start=1000000):
    s = rng.integers(-step, step + 1, n)
    return (start + np.cumsum(s)).astype(dtype)


def timestamps(rng, n):
    inc = rng.geometric(1 / 1000, n).astype(np.int64)
    out = rng.random(n) < 0.01
    inc[out] = rng.integers(0, 2**32, int(out.sum()))
    return (1700000000000000000 + np.cumsum(inc)).astype(np.int64)


def build_cases():
    rng = np.random.default_rng(20261203)
    c = []
    # the 1 MiB u32 random walk of the small numeric workload
    c.append(("walk_u32_1mib_dz_tsplit_fse", 1, walk(rng, 262144, np.uint32, 100), 4))
    c.append(("ts_i64_dz_bitpack_huf", 2, timestamps(rng, 100000), 8))
    for w, dt in [(1, np.uint8), (2, np.uint16), (4, np.uint32), (8, np.uint64)]:
        c.append(("walk_u%d_d_tsplit_fse" % (8 * w), 3, walk(rng, 70000 + 13 * w, dt, 3000), w))
        c.append(("walk_u%d_d_bitpack_huf" % (8 * w), 4, walk(rng, 70001 + 7 * w, dt, 300), w))
        c.append(("walk_u%d_delta_store" % (8 * w), 9, walk(rng, 5000 + w, dt, 100), w))
        c.append(("walk_u%d_zigzag_store" % (8 * w), 10, walk(rng, 4000 + w, dt, 100), w))
        c.append(("walk_u%d_bitpack_store" % (8 * w), 11, walk(rng, 3000 + w, dt, 100, start=500), w))
        c.append(("walk_u%d_tsplit_store" % (8 * w), 12, walk(rng, 3333 + w, dt, 100), w))
    keys = rng.integers(-2**31, 2**31, 10000).astype(np.int32)
    z = (rng.zipf(1.1, 200000) - 1) % 10000
    c.append(("tokenize_zipf_i32", 5, keys[z], 4))
    c.append(("tokenize_small_alphabet_i32", 5, rng.choice(keys[:200], 50000), 4))
    c.append(("tokenize_sorted_i32", 16, keys[z[:60000]], 4))
    bf = rng.normal(0, 0.02, 300000).astype(np.float32).view(np.uint32)
    c.append(("bf16_weights", 6, ((bf + 0x7FFF + ((bf >> 16) & 1)) >> 16).astype(np.uint16), 2))
    c.append(("fse_serial_skewed", 7, (rng.zipf(1.3, 300000) % 256).astype(np.uint8), 0))
    c.append(("fse_serial_small", 7, rng.integers(0, 4, 700).astype(np.uint8), 0))
    c.append(("huf_serial_skewed", 8, (rng.zipf(1.3, 300000) % 256).astype(np.uint8), 0))
    c.append(("huf_serial_uniform", 8, rng.integers(0, 256, 150000).astype(np.uint8), 0))
    c.append(("huf_serial_1x", 8, rng.integers(0, 6, 900).astype(np.uint8), 0))
    c.append(("constant_serial", 13, np.full(5000, 7, np.uint8), 0))
    c.append(("flatpack_serial", 14, rng.integers(0, 37, 30000).astype(np.uint8), 0))
    c.append(("bitpack_graph_serial", 15, rng.integers(0, 37, 30000).astype(np.uint8), 0))
    c.append(("store_serial", 0, rng.integers(0, 256, 3000).astype(np.uint8), 0))
    c.append(("empty_serial_fse", 7, np.zeros(0, np.uint8), 0))
    c.append(("tiny_numeric_delta", 9, np.array([5], np.uint32), 4))
    # 16-bit-symbol Huffman (huffman_struct_v2): u16 columns whose alphabet is
    # too wide for tokenize, through ZL_GRAPH_HUFFMAN
    c.append(("huf16_zipf_u16", 8, (rng.zipf(1.3, 200000) % 3000).astype(np.uint16), 2))
    c.append(("huf16_x1_u16", 8, (rng.zipf(1.2, 900) % 1000).astype(np.uint16), 2))
    c.append(("huf16_wide_u16", 8, np.minimum(rng.geometric(1 / 3000, 150000), 65535).astype(np.uint16), 2))
    # ZL_GRAPH_ENTROPY (EBM_any): per chunk FSE, Huffman, flatpack, bitpack,
    # constant or store
    lowent = np.where(rng.random(260000) < 0.98, 0, rng.integers(1, 256, 260000)).astype(np.uint8)
    c.append(("entropy_serial_lowent_fse", 17, lowent, 0))
    c.append(("entropy_serial_skewed_huf", 17, (rng.zipf(1.3, 300000) % 256).astype(np.uint8), 0))
    c.append(("entropy_serial_geom_mixed", 17, np.minimum(rng.geometric(0.2, 250000), 255).astype(np.uint8), 0))
    c.append(("entropy_serial_small_alpha", 17, rng.integers(0, 37, 30000).astype(np.uint8), 0))
    c.append(("entropy_serial_uniform_store", 17, rng.integers(0, 256, 50000).astype(np.uint8), 0))
    # older wire formats, written by the reference at a pinned format version
    # (decode-only: the encoders here write the newest version). Versions
    # 16..20 differ from 21+ in the frame and block headers only; 15 also
    # lacks the per-decoder regenerated-stream counts; 14 has no output
    # count; 8..13 have untyped outputs (serial only) and byte-sized block
    # counts before 9. Entropy-coded frames start at 15 (fse_v2/huffman_v2).
    for v in (20, 16, 15):
        c.append(("v%d_walk_u32_dz_tsplit_fse" % v, 1, walk(rng, 20000, np.uint32, 100), 4, True, v))
        c.append(("v%d_ts_i64_dz_bitpack_huf" % v, 2, timestamps(rng, 6000), 8, True, v))
        c.append(("v%d_walk_u16_d_tsplit_fse" % v, 3, walk(rng, 15001, np.uint16, 3000), 2, True, v))
        c.append(("v%d_walk_u64_d_bitpack_huf" % v, 4, walk(rng, 4003, np.uint64, 300), 8, True, v))
        c.append(("v%d_tokenize_zipf_i32" % v, 5, keys[(rng.zipf(1.1, 20000) - 1) % 10000], 4, True, v))
        c.append(("v%d_fse_serial_skewed" % v, 7, (rng.zipf(1.3, 20000) % 256).astype(np.uint8), 0, True, v))
        c.append(("v%d_huf_serial_skewed" % v, 8, (rng.zipf(1.3, 20000) % 256).astype(np.uint8), 0, True, v))
        c.append(("v%d_huf16_zipf_u16" % v, 8, (rng.zipf(1.3, 12000) % 3000).astype(np.uint16), 2, True, v))
        c.append(("v%d_entropy_serial_geom" % v, 17, np.minimum(rng.geometric(0.2, 20000), 255).astype(np.uint8), 0, True, v))
        c.append(("v%d_walk_u32_zigzag_store" % v, 10, walk(rng, 3001, np.uint32, 100), 4, True, v))
    for v in (14, 13, 9, 8):
        if v == 14:
            c.append(("v14_walk_u32_delta_store", 9, walk(rng, 3002, np.uint32, 100), 4, True, v))
            c.append(("v14_walk_u16_bitpack_store", 11, walk(rng, 2001, np.uint16, 100, start=500), 2, True, v))
            c.append(("v14_walk_u64_tsplit_store", 12, walk(rng, 1003, np.uint64, 100), 8, True, v))
        if v >= 11:
            c.append(("v%d_constant_serial" % v, 13, np.full(3000, 9, np.uint8), 0, True, v))
        c.append(("v%d_flatpack_serial" % v, 14, rng.integers(0, 37, 9000).astype(np.uint8), 0, True, v))
        c.append(("v%d_bitpack_graph_serial" % v, 15, rng.integers(0, 21, 9000).astype(np.uint8), 0, True, v))
        c.append(("v%d_store_serial" % v, 0, rng.integers(0, 256, 1500).astype(np.uint8), 0, True, v))
    # numbers through the constant graph (converted to struct first)
    for w, dt in [(2, np.uint16), (4, np.uint32), (8, np.uint64)]:
        c.append(("constant_u%d" % (8 * w), 13, np.full(4000 + w, 0x0102030405060708 % (256 ** w), dt), w))
    # Huffman histograms with a group of symbols of count 164, whose order
    # the reference's sort decides (candidates 1 and 7 of the generator; in
    # these the group straddles a code-length boundary)
    eq = equal_count_inputs(8)
    c.append(("huf_equal_counts_a", 8, eq[1], 0))
    c.append(("huf_equal_counts_b", 8, eq[7], 0))
    return c


def equal_count_inputs(n):
    """Serial inputs with 9 to 29 symbols of count 164 beside up to five
    large counts and 20 to 150 counts of 60 to 239 (seeded, shuffled)."""
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
        arr = np.concatenate([np.full(cnt, s, np.uint8) for s, cnt in counts.items()])
        rng.shuffle(arr)
        out.append(arr)
    return out


def build_multi_cases():
    """Frames of several inputs (ZL_CCtx_compressMultiTypedRef), each input
    through its own recipe graph; decode-only. (name, [(recipe, array,
    elt_width)], format version)."""
    rng = np.random.default_rng(20261204)
    c = []
    c.append(("multi2_fse_num_huf_serial", [(1, walk(rng, 20000, np.uint32, 100), 4),
                                            (8, (rng.zipf(1.3, 15000) % 256).astype(np.uint8), 0)], 0))
    c.append(("multi3_ts_delta_flatpack", [(2, timestamps(rng, 5000), 8), (9, walk(rng, 3000, np.uint16, 50), 2),
                                           (14, rng.integers(0, 37, 4000).astype(np.uint8), 0)], 0))
    c.append(("multi5_small_inputs", [(0, rng.integers(0, 256, 3).astype(np.uint8), 0),
                                      (10, walk(rng, 2, np.uint32, 9), 4),
                                      (7, (rng.zipf(1.3, 2000) % 40).astype(np.uint8), 0),
                                      (12, walk(rng, 700, np.uint64, 30), 8),
                                      (13, np.full(900, 5, np.uint8), 0)], 0))
    c.append(("multi16_extended_count", [(9 if k % 2 else 4, walk(rng, 500 + 37 * k, np.uint32, 60), 4)
                                         for k in range(16)], 0))
    c.append(("multi3_v20", [(1, walk(rng, 9000, np.uint16, 300), 2), (8, (rng.zipf(1.2, 6000) % 200).astype(np.uint8), 0),
                             (11, walk(rng, 1000, np.uint32, 40, start=900), 4)], 20))
    c.append(("multi4_huf16_entropy", [(8, (rng.zipf(1.3, 30000) % 3000).astype(np.uint16), 2),
                                       (17, np.minimum(rng.geometric(0.2, 20000), 255).astype(np.uint8), 0),
                                       (3, walk(rng, 40000, np.uint8, 3), 1),
                                       (5, rng.integers(0, 2**31, 500).astype(np.int32)[(rng.zipf(1.1, 9000) - 1) % 500], 4)],
                0))
    return c


def make_multi(lib):
    f = lib.ref_compress_multi
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    manifest = []
    for name, inputs, version in build_multi_cases():
        arrs = [np.ascontiguousarray(a) for _, a, _ in inputs]
        nb = len(inputs)
        for cs in (1, 0):
            rec = (ctypes.c_int * nb)(*[r for r, _, _ in inputs])
            srcs = (ctypes.c_void_p * nb)(*[a.ctypes.data for a in arrs])
            ns = (ctypes.c_size_t * nb)(*[a.size if w else a.nbytes for (_, _, w), a in zip(inputs, arrs)])
            ws = (ctypes.c_int * nb)(*[w for _, _, w in inputs])
            cap = sum(a.nbytes for a in arrs) * 2 + 8192 * nb
            dst = np.zeros(cap, np.uint8)
            r = f(nb, rec, srcs, ns, ws, dst.ctypes.data, cap, cs, version)
            if r <= 0:
                print("skip", name, cs, r)
                continue
            case = name + ("" if cs else "_nock")
            with open(os.path.join(HERE, case + ".zl"), "wb") as fh:
                fh.write(dst[:r].tobytes())
            manifest.append({"case": case, "checksums": cs, "frame_bytes": int(r),
                             "sha256_frame": hashlib.sha256(dst[:r].tobytes()).hexdigest(),
                             **({"format_version": version} if version else {}),
                             "outputs": [{"recipe": rr, "elt_width": w, "n": int(a.size), "type": 1 if w == 0 else 4,
                                          "bytes": int(a.nbytes), "sha256": hashlib.sha256(a.tobytes()).hexdigest()}
                                         for (rr, _, w), a in zip(inputs, arrs)]})
    manifest += make_strings(lib)
    with open(os.path.join(HERE, "manifest_multi.json"), "w") as fh:
        json.dump(manifest, fh, indent=1)
    return manifest


def make_strings(lib):
    """String inputs (one string output per frame): stored, FSE content with
    stored lengths, Huffman content with delta/bitpack/Huffman lengths."""
    f = lib.ref_compress_string
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                  ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    rng = np.random.default_rng(20261205)
    words = [bytes(rng.integers(97, 123, int(rng.integers(0, 14))).astype(np.uint8)) for _ in range(400)]
    out = []
    for name, recipe, nstr, version in (("str_store", 100, 3000, 0), ("str_fse_content", 101, 8000, 0),
                                        ("str_huf_content_coded_lens", 102, 20000, 0),
                                        ("str_huf_content_v21", 102, 5000, 21), ("str_empty_strings", 100, 50, 0)):
        pick = (rng.zipf(1.2, nstr) - 1) % len(words)
        strs = [words[i] if name != "str_empty_strings" else b"" for i in pick]
        content = np.frombuffer(b"".join(strs) + b"", np.uint8).copy()
        lens = np.array([len(x) for x in strs], np.uint32)
        for cs in (1, 0):
            cap = content.size * 2 + lens.nbytes * 2 + 65536
            dst = np.zeros(cap, np.uint8)
            r = f(recipe, content.ctypes.data if content.size else None, content.size, lens.ctypes.data, lens.size,
                  dst.ctypes.data, cap, cs, version)
            if r <= 0:
                print("skip", name, cs, r)
                continue
            case = name + ("" if cs else "_nock")
            with open(os.path.join(HERE, case + ".zl"), "wb") as fh:
                fh.write(dst[:r].tobytes())
            out.append({"case": case, "checksums": cs, "frame_bytes": int(r),
                        "sha256_frame": hashlib.sha256(dst[:r].tobytes()).hexdigest(),
                        **({"format_version": version} if version else {}),
                        "outputs": [{"recipe": recipe, "elt_width": 0, "n": int(lens.size), "type": 8,
                                     "bytes": int(content.size), "sha256": hashlib.sha256(content.tobytes()).hexdigest(),
                                     "sha256_lens": hashlib.sha256(lens.astype("<u4").tobytes()).hexdigest()}]})
    return out


def main():
    subprocess.check_call(["make", "-s", "-f", "oracle/ref.mk", "-j8"], cwd=ROOT)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "ref_driver.so"))
    lib.ref_compress.restype = ctypes.c_int64
    lib.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    lib.ref_compressBound.restype = ctypes.c_size_t
    manifest = []
    for name, recipe, arr, w, *flags in build_cases():
        decode_only = bool(flags and flags[0])
        version = flags[1] if len(flags) > 1 else 0  # 0: the newest format
        arr = np.ascontiguousarray(arr)
        for cs in (1, 0):
            if cs == 0 and recipe not in (1, 2, 3, 4, 5):
                continue
            cap = lib.ref_compressBound(arr.nbytes) + 4096
            dst = np.zeros(cap, np.uint8)
            n = arr.size if w else arr.nbytes
            r = lib.ref_compress(recipe, arr.ctypes.data if arr.size else None, n, w, dst.ctypes.data, cap, cs,
                                 version)
            if r <= 0:
                print("skip", name, cs, r)
                continue
            case = name + ("" if cs else "_nock")
            with open(os.path.join(HERE, case + ".zl"), "wb") as f:
                f.write(dst[:r].tobytes())
            manifest.append({"case": case, "recipe": recipe, "elt_width": w, "n": int(arr.size),
                             "checksums": cs, "frame_bytes": int(r),
                             "sha256_in": hashlib.sha256(arr.tobytes()).hexdigest(),
                             "sha256_frame": hashlib.sha256(dst[:r].tobytes()).hexdigest(),
                             **({"decode_only": True} if decode_only else {}),
                             **({"format_version": version} if version else {})})
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    multi = make_multi(lib)
    print(len(multi), "multi-output cases")
    tot = sum(os.path.getsize(os.path.join(HERE, m["case"] + ".zl")) for m in manifest)
    print(len(manifest), "cases,", tot, "bytes")


if __name__ == "__main__":
    sys.exit(main())
