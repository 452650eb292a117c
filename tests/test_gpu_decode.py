"""GPU decoder parity: every golden reference frame decodes byte-identically
to the reference's input (recorded hash) and to the CPU oracle, through the
host API, the device API and the batched CUDA-graph API."""
import hashlib

import numpy as np
import pytest

from conftest import read_frame
from oracle import oracle

pytestmark = pytest.mark.gpu


def _dev(torch, data, pad=64):
    """Device copy of bytes with slack after the end (the batch API's contract)."""
    b = np.frombuffer(data, np.uint8)
    t = torch.zeros(len(b) + pad, dtype=torch.uint8, device="cuda")
    if len(b):
        t[: len(b)].copy_(torch.from_numpy(b.copy()))
    return t


def test_host_api_golden(gpu_lib, manifest):
    import openzl_gb300 as oz

    d = oz.DCtx()
    for m in manifest:
        fr = read_frame(m["case"])
        out = d.decompress(fr)
        assert hashlib.sha256(out.tobytes()).hexdigest() == m["sha256_in"], m["case"]
        ref, _, _ = oracle.decompress(fr)
        assert out.tobytes() == ref.tobytes(), m["case"]


def test_device_api_golden(gpu_lib, manifest):
    import torch
    import openzl_gb300 as oz

    d = oz.DCtx()
    stream = torch.cuda.current_stream().cuda_stream
    for m in manifest:
        fr = read_frame(m["case"])
        n = oz.get_decompressed_size(fr)
        dfr = _dev(torch, fr)
        out = torch.empty(max(n, 1), dtype=torch.uint8, device="cuda")
        got = d.decompress_device(fr, dfr.data_ptr(), out.data_ptr(), n, stream)
        assert got == n
        h = hashlib.sha256(out[:n].cpu().numpy().tobytes()).hexdigest()
        assert h == m["sha256_in"], m["case"]


@pytest.mark.parametrize("graph", [False, True])
def test_batch_all_golden(gpu_lib, manifest, graph):
    import torch
    import openzl_gb300 as oz

    frames = [read_frame(m["case"]) for m in manifest]
    dfr = [_dev(torch, f) for f in frames]
    sizes = [oz.get_decompressed_size(f) for f in frames]
    outs = [torch.full((max(s, 1),), 0xAB, dtype=torch.uint8, device="cuda") for s in sizes]
    b = oz.GpuBatch()
    total = b.plan(frames, [t.data_ptr() for t in dfr], [o.data_ptr() for o in outs], sizes)
    assert total == sum(sizes)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()  # graph capture needs a non-default stream
    stream = side.cuda_stream
    for rep in range(2):
        b.run(stream, graph=graph)
        b.check(stream)
        for m, o, s in zip(manifest, outs, sizes):
            h = hashlib.sha256(o[:s].cpu().numpy().tobytes()).hexdigest()
            assert h == m["sha256_in"], (m["case"], rep)
        for o in outs:
            o.fill_(0xAB)
    assert b.launches() > 0


def test_corrupted_payload_reports_checksum_error(gpu_lib, manifest):
    import openzl_gb300 as oz

    m = next(m for m in manifest if m["case"] == "walk_u32_1mib_dz_tsplit_fse")
    fr = bytearray(read_frame(m["case"]))
    fr[len(fr) // 2] ^= 0x01  # inside a stored FSE bitstream
    with pytest.raises(oz.ZLError) as e:
        oz.DCtx().decompress(bytes(fr))
    assert e.value.code in (12, 13, 14)


def test_truncated_frame_is_rejected_on_host(gpu_lib):
    import openzl_gb300 as oz

    fr = read_frame("ts_i64_dz_bitpack_huf")
    with pytest.raises(oz.ZLError):
        oz.DCtx().decompress(fr[: len(fr) // 3])


def test_device_api_side_stream_back_to_back(gpu_lib):
    """Many frames of growing size decoded one call after another on a
    non-blocking stream: each call's plan upload is ordered before its own
    kernels (a plan uploaded off-stream raced the next frame's launch)."""
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(5)
    s = torch.cuda.Stream()
    d = oz.DCtx()
    cases = []
    for k in range(24):
        n = int(2000 * 1.5 ** k) // 8 + 1
        a = (1000 + np.cumsum(rng.integers(-300, 301, n))).astype(np.uint32)
        recipe = 3 if k % 2 else 4
        cases.append((a, oracle.compress(recipe, a, 4)))
    dfr = [_dev(torch, f.tobytes()) for _, f in cases]
    outs = [torch.zeros(a.nbytes + 64, dtype=torch.uint8, device="cuda") for a, _ in cases]
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        for (a, f), df, o in zip(cases, dfr, outs):
            d.decompress_device(f, df.data_ptr(), o.data_ptr(), a.nbytes, s.cuda_stream)
    s.synchronize()
    for (a, _), o in zip(cases, outs):
        assert o[: a.nbytes].cpu().numpy().tobytes() == a.tobytes()


def test_autotuned_shapes_keep_results(gpu_lib, manifest):
    """The autotuner changes only launch shapes: the batch decodes the same
    bytes before and after, through the captured graph."""
    import torch
    import openzl_gb300 as oz

    frames = [read_frame(m["case"]) for m in manifest]
    dfr = [_dev(torch, f) for f in frames]
    sizes = [oz.get_decompressed_size(f) for f in frames]
    outs = [torch.zeros(max(n, 1) + 64, dtype=torch.uint8, device="cuda") for n in sizes]
    s = torch.cuda.Stream()
    b = oz.GpuBatch()
    b.plan(frames, [d.data_ptr() for d in dfr], [o.data_ptr() for o in outs], sizes)
    torch.cuda.synchronize()
    shapes = b.autotune(s.cuda_stream, reps=1)
    assert len(shapes) > 0 and any(x > 0 for x in shapes)
    for o in outs:
        o.zero_()
    torch.cuda.synchronize()
    b.run(s.cuda_stream, graph=True)
    b.check(s.cuda_stream)
    for m, n, o in zip(manifest, sizes, outs):
        h = hashlib.sha256(o[:n].cpu().numpy().tobytes()).hexdigest()
        assert h == m["sha256_in"], m["case"]


def _layout(sizes, align):
    offs, o = [], 0
    for s in sizes:
        offs.append(o)
        o += (s + align - 1) // align * align
    return offs, o


@pytest.mark.parametrize("graph", [False, True])
def test_batch_run_host_pipelined(gpu_lib, manifest, graph):
    """ozl_gpu_batch_run_host with host images of frames and outputs laid out
    in order: the copies in, the decode and the copies out run in overlapped
    rounds, and the host output equals the reference's inputs; frames whose
    addresses do not increase with their index take the serial path with the
    same result; a corrupted frame is reported."""
    import torch
    import openzl_gb300 as oz

    frames = [read_frame(m["case"]) for m in manifest] * 3
    want = [m["sha256_in"] for m in manifest] * 3
    sizes = [oz.get_decompressed_size(f) for f in frames]
    foffs, fbytes = _layout([len(f) for f in frames], 16)
    ooffs, obytes = _layout([max(s, 1) for s in sizes], 256)
    fbytes += 64
    h_in = torch.zeros(fbytes, dtype=torch.uint8, pin_memory=True)
    for f, o in zip(frames, foffs):
        h_in[o:o + len(f)].copy_(torch.from_numpy(np.frombuffer(f, np.uint8).copy()))
    d_in = torch.zeros(fbytes, dtype=torch.uint8, device="cuda")
    d_out = torch.zeros(obytes, dtype=torch.uint8, device="cuda")
    h_out = torch.zeros(obytes, dtype=torch.uint8, pin_memory=True)
    s = torch.cuda.Stream()
    for order in ("increasing", "swapped"):
        idx = list(range(len(frames)))
        if order == "swapped":
            # frames 1 and 2 planned in swapped order: the image still starts
            # at the first frame, but the addresses no longer increase
            idx[1], idx[2] = idx[2], idx[1]
        b = oz.GpuBatch()
        b.plan([frames[i] for i in idx], [d_in.data_ptr() + foffs[i] for i in idx],
               [d_out.data_ptr() + ooffs[i] for i in idx], [sizes[i] for i in idx])
        for rep in range(4):
            h_out.fill_(0xAB)
            if rep == 3:  # the timeline run: rounds (in order) or none (serial path)
                rows = b.host_timeline(h_in.data_ptr(), fbytes, h_out.data_ptr(), obytes, s.cuda_stream)
                if order == "increasing":
                    assert len(rows) > 1 and all(a <= c and d <= c for a, d, c in rows), rows
                else:
                    assert rows == []
                    b.run_host(h_in.data_ptr(), fbytes, h_out.data_ptr(), obytes, s.cuda_stream, graph=graph)
            else:
                b.run_host(h_in.data_ptr(), fbytes, h_out.data_ptr(), obytes, s.cuda_stream, graph=graph)
            for i in range(len(frames)):
                got = h_out[ooffs[i]:ooffs[i] + sizes[i]].numpy().tobytes()
                assert hashlib.sha256(got).hexdigest() == want[i], (order, rep, i)
    # a corrupted payload byte in one frame of the image is reported
    b = oz.GpuBatch()
    b.plan(frames, [d_in.data_ptr() + o for o in foffs], [d_out.data_ptr() + o for o in ooffs], sizes)
    k = next(i for i, m in enumerate(manifest) if m["case"] == "walk_u32_1mib_dz_tsplit_fse")
    bad = h_in.clone().pin_memory()
    bad[foffs[k] + len(frames[k]) // 2] ^= 0x01  # inside a stored FSE bitstream
    with pytest.raises(oz.ZLError):
        b.run_host(bad.data_ptr(), fbytes, h_out.data_ptr(), obytes, s.cuda_stream, graph=graph)


def test_huffman16_frames_run_the_16bit_kernel(gpu_lib, manifest):
    """The 16-bit-symbol Huffman fixtures (huffman_struct_v2, transform 51)
    decode through the GPU's 16-bit Huffman launch, bit-exactly."""
    import torch
    import openzl_gb300 as oz

    cases = [m for m in manifest if m["case"].startswith("huf16_")]
    assert len(cases) >= 3
    frames = [read_frame(m["case"]) for m in cases]
    dfr = [_dev(torch, f) for f in frames]
    sizes = [oz.get_decompressed_size(f) for f in frames]
    outs = [torch.zeros(max(n, 1) + 64, dtype=torch.uint8, device="cuda") for n in sizes]
    s = torch.cuda.Stream()
    b = oz.GpuBatch()
    b.plan(frames, [d.data_ptr() for d in dfr], [o.data_ptr() for o in outs], sizes)
    torch.cuda.synchronize()
    kinds = [k for k, _, _ in b.profile(s.cuda_stream, capacity=64)]
    assert "huffman16" in kinds, kinds
    b.run(s.cuda_stream, graph=True)
    b.check(s.cuda_stream)
    for m, n, o in zip(cases, sizes, outs):
        assert hashlib.sha256(o[:n].cpu().numpy().tobytes()).hexdigest() == m["sha256_in"], m["case"]


def test_older_format_versions_on_the_gpu(gpu_lib, manifest):
    """Frames of format versions 8..20 decode bit-exactly through the batch
    API, with their checksums verified on the device; a payload byte flipped
    in a v20 frame fails the compressed checksum, which before v21 spans the
    frame from its first byte."""
    import torch
    import openzl_gb300 as oz

    cases = [m for m in manifest if m.get("format_version", 23) < 21]
    assert len(cases) >= 40
    frames = [read_frame(m["case"]) for m in cases]
    dfr = [_dev(torch, f) for f in frames]
    sizes = [oz.get_decompressed_size(f) for f in frames]
    outs = [torch.zeros(max(n, 1) + 64, dtype=torch.uint8, device="cuda") for n in sizes]
    s = torch.cuda.Stream()
    b = oz.GpuBatch()
    b.plan(frames, [d.data_ptr() for d in dfr], [o.data_ptr() for o in outs], sizes)
    torch.cuda.synchronize()
    kinds = {k for k, _, _ in b.profile(s.cuda_stream, capacity=256)}
    assert {"fse", "huffman", "huffman16"} <= kinds, kinds
    b.run(s.cuda_stream, graph=True)
    b.check(s.cuda_stream)
    for m, n, o in zip(cases, sizes, outs):
        assert hashlib.sha256(o[:n].cpu().numpy().tobytes()).hexdigest() == m["sha256_in"], m["case"]
    fr = bytearray(read_frame("v20_walk_u32_dz_tsplit_fse"))
    fr[len(fr) // 2] ^= 0x01
    with pytest.raises(oz.ZLError) as e:
        oz.DCtx().decompress(bytes(fr))
    assert e.value.code in (12, 13, 14)


def test_multi_output_frames(gpu_lib, manifest, manifest_multi):
    """Frames of several outputs: ZL_DCtx_decompressMultiTBuffer returns each
    output with its type and width; the batch API, mixed with single-output
    frames, writes each output at the offset ozl_frame_outputs gives (content
    checksums over the gathered outputs verified on the device); a corrupted
    frame and a wrong output count are reported."""
    import torch
    import openzl_gb300 as oz

    d = oz.DCtx()
    for m in manifest_multi:
        outs = d.decompress_multi(read_frame(m["case"]), with_lengths=True)
        assert len(outs) == len(m["outputs"]), m["case"]
        for (data, t, w, lens), o in zip(outs, m["outputs"]):
            assert hashlib.sha256(data.tobytes()).hexdigest() == o["sha256"], m["case"]
            assert t == o["type"] and w == (o["elt_width"] or 1), m["case"]
            if t == 8:
                assert hashlib.sha256(lens.astype("<u4").tobytes()).hexdigest() == o["sha256_lens"], m["case"]
    singles = manifest[:8]
    frames = [read_frame(m["case"]) for m in manifest_multi] + [read_frame(m["case"]) for m in singles]
    layouts, extents = zip(*[oz.frame_outputs(f) for f in frames])
    dfr = [_dev(torch, f) for f in frames]
    outs = [torch.full((max(e, 1) + 64,), 0xAB, dtype=torch.uint8, device="cuda") for e in extents]
    s = torch.cuda.Stream()
    b = oz.GpuBatch()
    total = b.plan(frames, [x.data_ptr() for x in dfr], [o.data_ptr() for o in outs], extents)
    assert total == sum(extents)
    torch.cuda.synchronize()
    for graph in (False, True):
        b.run(s.cuda_stream, graph=graph)
        b.check(s.cuda_stream)
        for k, (lay, o) in enumerate(zip(layouts, outs)):
            host = o.cpu().numpy()
            want = manifest_multi[k]["outputs"] if k < len(manifest_multi) else [
                {"sha256": singles[k - len(manifest_multi)]["sha256_in"]}]
            for l, w in zip(lay, want):
                got = host[l["offset"]:l["offset"] + l["size"]].tobytes()
                assert hashlib.sha256(got).hexdigest() == w["sha256"], (k, graph)
                if l["type"] == 8:
                    lens = host[l["lens_offset"]:l["lens_offset"] + 4 * l["count"]].tobytes()
                    assert hashlib.sha256(lens).hexdigest() == w["sha256_lens"], (k, graph)
    m = next(m for m in manifest_multi if m["case"] == "multi3_ts_delta_flatpack")
    bad = bytearray(read_frame(m["case"]))
    bad[len(bad) // 2] ^= 0x01
    with pytest.raises(oz.ZLError):
        d.decompress_multi(bytes(bad))
    # the content checksum of a multi-output block covers its gathered
    # outputs: flip a byte of it and decode without the compressed checksum
    # (which covers the content checksum too)
    fr = read_frame("multi3_ts_delta_flatpack")
    bad = bytes(fr[:-6]) + bytes([fr[-6] ^ 0x10]) + bytes(fr[-5:])  # content, compressed checksums, end marker
    lay, ext = oz.frame_outputs(fr)
    dbad = _dev(torch, bad)
    o = torch.zeros(ext + 64, dtype=torch.uint8, device="cuda")
    bb = oz.GpuBatch(check_compressed=False)
    bb.plan([bad], [dbad.data_ptr()], [o.data_ptr()], [ext])
    torch.cuda.synchronize()
    bb.run(s.cuda_stream, graph=False)
    with pytest.raises(oz.ZLError) as e:
        bb.check(s.cuda_stream)
    assert e.value.code == 14
    fr = read_frame("multi5_small_inputs")
    import ctypes
    lib = oz.library()
    arr = (ctypes.c_void_p * 1)(lib.ZL_TypedBuffer_create())
    f = np.frombuffer(fr, np.uint8)
    rep = lib.ZL_DCtx_decompressMultiTBuffer(d._h, arr, 1, f.ctypes.data, f.size)
    lib.ZL_TypedBuffer_free(arr[0])
    assert rep.code == 8


@pytest.mark.parametrize("parts_per_kind,critical,schedule",
                         [(1, 0, 0), (2, 0, 0), (4, 0, 0), (1, 1000, 0), (2, 16000, 0), (8, 100, 0), (2, 16000, 1)])
def test_batch_parts_per_kind_keep_results(gpu_lib, manifest, parts_per_kind, critical, schedule):
    """Runs of frames decoded as parallel graph branches at falling stream
    priorities (each kind split into 1 to 8 runs; frames with an FSE stream of
    at least `critical` symbols as one more branch, 17 branches at most) give
    the same bytes, with and without the graph."""
    import torch
    import openzl_gb300 as oz

    frames = [read_frame(m["case"]) for m in manifest]
    dfr = [_dev(torch, f) for f in frames]
    sizes = [oz.get_decompressed_size(f) for f in frames]
    outs = [torch.zeros(max(n, 1) + 64, dtype=torch.uint8, device="cuda") for n in sizes]
    s = torch.cuda.Stream()
    b = oz.GpuBatch(parts_per_kind=parts_per_kind, critical_symbols=critical, schedule=schedule)
    b.plan(frames, [d.data_ptr() for d in dfr], [o.data_ptr() for o in outs], sizes)
    torch.cuda.synchronize()
    for graph in (False, True):
        for o in outs:
            o.zero_()
        b.run(s.cuda_stream, graph=graph)
        b.check(s.cuda_stream)
        for m, n, o in zip(manifest, sizes, outs):
            assert hashlib.sha256(o[:n].cpu().numpy().tobytes()).hexdigest() == m["sha256_in"], (m["case"], graph)
    # the timeline run: one row per planned launch, each ending after its
    # stream reached it, and the same bytes
    for o in outs:
        o.zero_()
    rows = b.timeline(s.cuda_stream)
    b.check(s.cuda_stream)
    assert rows and all(end >= start for _, _, _, start, end in rows), rows[:4]
    assert len({part for part, _, _, _, _ in rows}) >= 1
    for m, n, o in zip(manifest, sizes, outs):
        assert hashlib.sha256(o[:n].cpu().numpy().tobytes()).hexdigest() == m["sha256_in"], m["case"]


def test_huffman_tablelog12_chunks(gpu_lib):
    """Huffman chunks at table log 12 (a table across two slots, decoded in a
    second round of the CTA) through the host API and the batch API, before
    and after the autotuner (CTAs of 2 to 8 chunks), against the input."""
    import torch
    import openzl_gb300 as oz
    from test_oracle import huf_tablelog12_cases

    cases = huf_tablelog12_cases()
    d = oz.DCtx()
    for recipe, arr, w, fr in cases:
        out = d.decompress_typed(fr.tobytes())[0] if w else d.decompress(fr.tobytes())
        assert out.tobytes() == arr.tobytes(), (recipe, arr.size)
    frames = [fr.tobytes() for _, _, _, fr in cases]
    dfr = [_dev(torch, f) for f in frames]
    outs = [torch.zeros(a.nbytes + 64, dtype=torch.uint8, device="cuda") for _, a, _, _ in cases]
    b = oz.GpuBatch()
    b.plan(frames, [t.data_ptr() for t in dfr], [o.data_ptr() for o in outs], [a.nbytes for _, a, _, _ in cases])
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    for tune in (False, True):
        if tune:
            b.autotune(side.cuda_stream, reps=1)
        for o in outs:
            o.zero_()
        b.run(side.cuda_stream, graph=True)
        b.check(side.cuda_stream)
        for (_, a, _, _), o in zip(cases, outs):
            assert o[:a.nbytes].cpu().numpy().tobytes() == a.tobytes(), tune


def test_fse_tablelog12_streams(gpu_lib):
    """FSE chunks at table log 12 (the widest fields and largest state bases
    of the four-state register-window loop), unchunked streams of 99,999
    symbols included: host API and batched API against the input."""
    import torch
    import openzl_gb300 as oz
    from test_oracle import tablelog12_cases

    cases = tablelog12_cases()
    d = oz.DCtx()
    for recipe, arr, w, fr in cases:
        out = d.decompress_typed(fr.tobytes())[0] if w else d.decompress(fr.tobytes())
        assert out.tobytes() == arr.tobytes(), (recipe, arr.size)
    frames = [fr.tobytes() for _, _, _, fr in cases]
    dfr = [_dev(torch, f) for f in frames]
    outs = [torch.zeros(a.nbytes + 64, dtype=torch.uint8, device="cuda") for _, a, _, _ in cases]
    b = oz.GpuBatch()
    b.plan(frames, [t.data_ptr() for t in dfr], [o.data_ptr() for o in outs], [a.nbytes for _, a, _, _ in cases])
    torch.cuda.synchronize()
    side = torch.cuda.Stream()  # graph capture needs a non-default stream
    b.run(side.cuda_stream, graph=True)
    b.check(side.cuda_stream)
    for (_, a, _, _), o in zip(cases, outs):
        assert o[:a.nbytes].cpu().numpy().tobytes() == a.tobytes()


@pytest.mark.parametrize("fse_kernel", [1, 2])
def test_fse_kernels_on_golden_and_tablelog12(gpu_lib, manifest, fse_kernel):
    """Both FSE decoders (one lane per stream; one lane per decoder state,
    four per stream) on every golden frame and on table-log-12 streams,
    through captured batch runs."""
    import torch
    import openzl_gb300 as oz
    from test_oracle import tablelog12_cases

    frames = [read_frame(m["case"]) for m in manifest]
    wants = [m["sha256_in"] for m in manifest]
    for _, a, _, fr in tablelog12_cases():
        frames.append(fr.tobytes())
        wants.append(hashlib.sha256(a.tobytes()).hexdigest())
    dfr = [_dev(torch, f) for f in frames]
    sizes = [oz.get_decompressed_size(f) for f in frames]
    outs = [torch.full((max(s, 1),), 0xAB, dtype=torch.uint8, device="cuda") for s in sizes]
    b = oz.GpuBatch(fse_kernel=fse_kernel)
    b.plan(frames, [t.data_ptr() for t in dfr], [o.data_ptr() for o in outs], sizes)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    for rep in range(2):
        b.run(side.cuda_stream, graph=True)
        b.check(side.cuda_stream)
        for w, o, s in zip(wants, outs, sizes):
            assert hashlib.sha256(o[:s].cpu().numpy().tobytes()).hexdigest() == w, rep


def test_fse_kernels_agree_on_random_walk_frames(gpu_lib):
    """Transpose-split FSE frames of every element width, sizes from a few
    symbols to several chunks, decoded with both FSE kernels: the same bytes,
    equal to the input."""
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(44)
    arrs, frames = [], []
    for k in range(60):
        w = [1, 2, 4, 8][k % 4]
        n = int(np.exp(rng.uniform(np.log(3), np.log(300000 // w))))
        a = (1000 + np.cumsum(rng.integers(-int(rng.integers(1, 60000)), 60000, n))).astype(
            {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[w])
        arrs.append(a)
        frames.append(oracle.compress(3, a, w).tobytes())
    dfr = [_dev(torch, f) for f in frames]
    got = {}
    for fk in (1, 2):
        outs = [torch.zeros(a.nbytes + 64, dtype=torch.uint8, device="cuda") for a in arrs]
        b = oz.GpuBatch(fse_kernel=fk)
        b.plan(frames, [t.data_ptr() for t in dfr], [o.data_ptr() for o in outs], [a.nbytes for a in arrs])
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        b.run(side.cuda_stream, graph=True)
        b.check(side.cuda_stream)
        got[fk] = [o[:a.nbytes].cpu().numpy().tobytes() for o, a in zip(outs, arrs)]
    for a, x, y in zip(arrs, got[1], got[2]):
        assert x == a.tobytes() and y == a.tobytes()
