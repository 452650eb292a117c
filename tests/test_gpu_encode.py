"""GPU encoder parity: frames compressed on the device are byte-identical to
the CPU oracle's (itself pinned to the reference's frames), and decode back
on the device to the input."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _walk(rng, n, dt, step, start=1000000):
    return (start + np.cumsum(rng.integers(-step, step + 1, n))).astype(dt)


def _timestamps(rng, n):
    inc = rng.geometric(1 / 1000, n).astype(np.int64)
    o = rng.random(n) < 0.01
    inc[o] = rng.integers(0, 2**32, int(o.sum()))
    return (1700000000000000000 + np.cumsum(inc)).astype(np.int64)


def _cases(seed):
    rng = np.random.default_rng(seed)
    c = [(1, _walk(rng, 262144, np.uint32, 100), 4), (2, _timestamps(rng, 150000), 8)]
    for w, dt in [(1, np.uint8), (2, np.uint16), (4, np.uint32), (8, np.uint64)]:
        for recipe in (1, 2, 3, 4, 9, 10, 11, 12):
            for n in (1, 3, 9, 700, 20000 + 17 * w, 130000):
                c.append((recipe, _walk(rng, n, dt, int(rng.integers(1, 6000))), w))
    for recipe in (7, 8):
        for n in (2, 9, 10, 999, 1001, 5000, 100000, 200000):
            for k in (2, 3, 37, 256):
                c.append((recipe, (rng.zipf(1.2, n) % k).astype(np.uint8), 0))
    keys = rng.integers(0, 2**31, 10000).astype(np.int32)
    for n in (3, 700, 20000, 300000):
        idx = (rng.zipf(1.1, n) - 1) % keys.size
        c.append((5, keys[idx].astype(np.uint32), 4))
    c.append((5, (rng.integers(0, 200, 50000)).astype(np.uint16), 2))
    # sorted alphabet (recipe 16): indices renumbered after a host sort
    for n in (3, 700, 20000, 300000):
        idx = (rng.zipf(1.1, n) - 1) % keys.size
        c.append((16, keys[idx].astype(np.uint32), 4))
    c.append((16, (rng.integers(0, 300, 50000)).astype(np.uint16), 2))
    c.append((16, (rng.integers(0, 2**40, 3000)).astype(np.uint64), 8))
    c.append((5, (rng.integers(0, 2**40, 3000)).astype(np.uint64), 8))
    for n in (4, 900, 70000):
        bf = (rng.normal(0, 0.02, n).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
        c.append((6, bf, 2))
    c.append((13, np.full(4000, 9, np.uint8), 0))
    c.append((14, rng.integers(0, 37, 3000).astype(np.uint8), 0))
    c.append((15, rng.integers(0, 37, 3000).astype(np.uint8), 0))
    # the entropy graph (FSE or Huffman per chunk)
    for n in (2, 999, 5000, 100000, 300000):
        for k in (3, 37, 256):
            c.append((17, (rng.zipf(1.2, n) % k).astype(np.uint8), 0))
        c.append((17, np.where(rng.random(n) < 0.98, 0, rng.integers(1, 256, n)).astype(np.uint8), 0))
    c.append((0, rng.integers(0, 256, 3000).astype(np.uint8), 0))
    # 2-byte input to the Huffman and entropy graphs: per chunk constant,
    # bit packing, store, tokenize (fewer than 256 values) or
    # huffman_struct_v2 (1 or 4 streams), chunked from 100000 elements
    for recipe in (8, 17):
        for n in (2, 3, 999, 1001, 40000, 140000):
            c.append((recipe, (rng.zipf(1.3, n) % 3000).astype(np.uint16), 2))
            c.append((recipe, (rng.zipf(1.2, n) % 200).astype(np.uint16), 2))
            c.append((recipe, np.minimum(rng.geometric(1 / 3000, n), 65535).astype(np.uint16), 2))
            c.append((recipe, rng.integers(0, 40, n).astype(np.uint16), 2))
        c.append((recipe, np.full(5000, 777, np.uint16), 2))
        c.append((recipe, rng.integers(0, 65536, 20000).astype(np.uint16), 2))
    return c


@pytest.mark.parametrize("checksums", [True, False])
def test_gpu_frames_equal_oracle_frames(gpu_lib, checksums):
    import torch
    import openzl_gb300 as oz

    cases = _cases(11 if checksums else 12)
    enc = oz.GpuEncoder()
    srcs = [torch.from_numpy(a.view(np.uint8).copy()).cuda() if a.size else torch.zeros(1, dtype=torch.uint8,
            device="cuda") for _, a, _ in cases]
    caps = [enc.bound(a.nbytes) for _, a, _ in cases]
    dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([s.data_ptr() for s in srcs], [a.size if w else a.nbytes for _, a, w in cases],
                               [w for _, _, w in cases], [r for r, _, _ in cases], [d.data_ptr() for d in dsts],
                               caps, checksums=checksums)
    bad = []
    for (recipe, arr, w), d, sz in zip(cases, dsts, sizes):
        want = oracle.compress(recipe, arr, w, checksums=checksums).tobytes()
        got = d[:sz].cpu().numpy().tobytes()
        if got != want:
            bad.append((recipe, w, arr.size, len(got), len(want)))
    assert not bad, bad[:10]


def test_fse_chunks_around_the_per_state_threshold(gpu_lib):
    """Serial inputs through the FSE graph: lengths around 4,096 symbols (from
    there a chunk's four states run on four lanes and a warp packs their
    fields), every length mod 4, around the 32 KiB chunks and the
    100,000-symbol chunking threshold; bytes from two symbols to all 256.
    Frames equal the oracle's byte for byte."""
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(4096)
    lengths = list(range(4092, 4101)) + [6001, 32767, 32768, 32769, 65539, 99999, 100000, 100001, 100003, 131074]
    cases = []
    for n in lengths:
        cases.append((rng.random(n) < 0.02).astype(np.uint8))                       # two symbols, skewed
        cases.append((rng.zipf(1.3, n) % 5).astype(np.uint8))
        cases.append((rng.zipf(1.1, n) % 256).astype(np.uint8))
        cases.append(np.minimum(rng.geometric(0.05, n), 255).astype(np.uint8))
        cases.append(rng.integers(0, 256, n).astype(np.uint8))                      # near uniform
    enc = oz.GpuEncoder()
    srcs = [torch.from_numpy(a.copy()).cuda() for a in cases]
    caps = [enc.bound(a.nbytes) for a in cases]
    dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([x.data_ptr() for x in srcs], [a.nbytes for a in cases], [0] * len(cases),
                               [7] * len(cases), [d.data_ptr() for d in dsts], caps, checksums=True)
    bad = [(k, a.size) for k, (a, d, sz) in enumerate(zip(cases, dsts, sizes))
           if d[:sz].cpu().numpy().tobytes() != oracle.compress(7, a, 0).tobytes()]
    assert not bad, bad[:10]


def test_huffman_equal_count_groups(gpu_lib):
    """Histograms with a group of symbols of count 164 (the reference's
    Huffman sort reorders them): GPU frames through the Huffman and entropy
    graphs equal the oracle's, which the CPU tests pin to the reference's."""
    import torch
    import openzl_gb300 as oz
    from test_oracle import equal_count_cases

    cases = [(r, a) for a in equal_count_cases() for r in (8, 17)]
    enc = oz.GpuEncoder()
    srcs = [torch.from_numpy(a.copy()).cuda() for _, a in cases]
    caps = [enc.bound(a.nbytes) for _, a in cases]
    dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([x.data_ptr() for x in srcs], [a.nbytes for _, a in cases], [0] * len(cases),
                               [r for r, _ in cases], [d.data_ptr() for d in dsts], caps, checksums=True)
    bad = [(k, r) for k, ((r, a), d, sz) in enumerate(zip(cases, dsts, sizes))
           if d[:sz].cpu().numpy().tobytes() != oracle.compress(r, a, 0).tobytes()]
    assert not bad, bad[:10]


def test_constant_graph(gpu_lib):
    """The constant graph: numbers of 1 to 8 bytes (converted to struct) and
    serial bytes give the oracle's frames; input that is not constant is
    refused, as the reference refuses it."""
    import torch
    import openzl_gb300 as oz
    from test_oracle import constant_graph_cases

    cases = constant_graph_cases()
    enc = oz.GpuEncoder()
    srcs = [torch.from_numpy(a.view(np.uint8).copy()).cuda() for a, _ in cases]
    caps = [enc.bound(a.nbytes) for a, _ in cases]
    dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([x.data_ptr() for x in srcs], [a.size if w else a.nbytes for a, w in cases],
                               [w for _, w in cases], [13] * len(cases), [d.data_ptr() for d in dsts], caps,
                               checksums=True)
    bad = [(k, w, a.size) for k, ((a, w), d, sz) in enumerate(zip(cases, dsts, sizes))
           if d[:sz].cpu().numpy().tobytes() != oracle.compress(13, a, w).tobytes()]
    assert not bad, bad
    for w, dt in [(0, np.uint8), (1, np.uint8), (2, np.uint16), (8, np.uint64)]:
        a = np.full(1000, 7, dt)
        a[500] = 8
        x = torch.from_numpy(a.view(np.uint8).copy()).cuda()
        d = torch.zeros(enc.bound(a.nbytes), dtype=torch.uint8, device="cuda")
        with pytest.raises(Exception):
            enc.compress_batch([x.data_ptr()], [a.size if w else a.nbytes], [w], [13], [d.data_ptr()],
                               [enc.bound(a.nbytes)], checksums=True)


def test_gpu_encode_then_gpu_decode(gpu_lib):
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(5)
    arrs = [(3, _walk(rng, 300000, np.uint16, 3000), 2), (4, _walk(rng, 250000, np.uint64, 60000), 8),
            (1, _walk(rng, 262144, np.uint32, 100), 4), (2, _timestamps(rng, 400000), 8)]
    enc = oz.GpuEncoder()
    srcs = [torch.from_numpy(a.view(np.uint8).copy()).cuda() for _, a, _ in arrs]
    caps = [enc.bound(a.nbytes) for _, a, _ in arrs]
    dsts = [torch.zeros(c + 64, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([s.data_ptr() for s in srcs], [a.size for _, a, _ in arrs], [w for _, _, w in arrs],
                               [r for r, _, _ in arrs], [d.data_ptr() for d in dsts], caps)
    d = oz.DCtx()
    for (_, a, _), dst, sz in zip(arrs, dsts, sizes):
        frame = dst[:sz].cpu().numpy()
        assert d.decompress(frame).tobytes() == a.tobytes()


def test_gpu_frames_equal_oracle_frames_many_frames(gpu_lib):
    """600 frames in one call: graph discovery, decisions and replay run on
    host threads (from 256 frames or jobs) and the frames stay identical to
    the oracle's."""
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(77)
    cases = []
    for k in range(600):
        recipe = (1, 2, 3, 4, 7, 8, 17, 9)[k % 8]
        n = int(rng.integers(2, 40000))
        if recipe in (7, 8, 17):
            cases.append((recipe, (rng.zipf(1.25, n) % int(rng.integers(2, 256))).astype(np.uint8), 0))
        else:
            dt, w = [(np.uint8, 1), (np.uint16, 2), (np.uint32, 4), (np.uint64, 8)][k % 4]
            cases.append((recipe, _walk(rng, n, dt, int(rng.integers(1, 3000))), w))
    enc = oz.GpuEncoder()
    srcs = [torch.from_numpy(a.view(np.uint8).copy()).cuda() for _, a, _ in cases]
    caps = [enc.bound(a.nbytes) for _, a, _ in cases]
    dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([s.data_ptr() for s in srcs], [a.size if w else a.nbytes for _, a, w in cases],
                               [w for _, _, w in cases], [r for r, _, _ in cases], [d.data_ptr() for d in dsts],
                               caps, checksums=True)
    bad = []
    for k, ((recipe, arr, w), d, sz) in enumerate(zip(cases, dsts, sizes)):
        if d[:sz].cpu().numpy().tobytes() != oracle.compress(recipe, arr, w).tobytes():
            bad.append((k, recipe, w, arr.size))
    assert not bad, bad[:10]


@pytest.mark.parametrize("parts", [1, 3, 8])
def test_encoder_parts_keep_frames(gpu_lib, parts):
    """A batch of 64 MiB or more runs in parts (each on its own host thread
    and stream); the frames equal the oracle's for every part count, and the
    phase times are reported."""
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(909)
    cases = []
    total = 0
    k = 0
    while total < (80 << 20):
        recipe = (3, 4, 1, 2, 8)[k % 5]
        n = int(rng.integers(100000, 700000))
        if recipe == 8:
            a = (rng.zipf(1.3, n) % 200).astype(np.uint8)
            cases.append((recipe, a, 0))
        else:
            dt, w = [(np.uint16, 2), (np.uint32, 4), (np.uint64, 8)][k % 3]
            a = _walk(rng, n, dt, int(rng.integers(1, 5000)))
            cases.append((recipe, a, w))
        total += a.nbytes
        k += 1
    enc = oz.GpuEncoder()
    enc.set_parts(parts)
    srcs = [torch.from_numpy(a.view(np.uint8).copy()).cuda() for _, a, _ in cases]
    caps = [enc.bound(a.nbytes) for _, a, _ in cases]
    dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
    sizes = enc.compress_batch([s.data_ptr() for s in srcs], [a.size if w else a.nbytes for _, a, w in cases],
                               [w for _, _, w in cases], [r for r, _, _ in cases], [d.data_ptr() for d in dsts],
                               caps, checksums=True)
    ph = enc.phases()
    assert set(ph) == set(oz.GpuEncoder.PHASES) and all(v >= 0 for v in ph.values()) and sum(ph.values()) > 0
    bad = [k for k, ((recipe, arr, w), d, sz) in enumerate(zip(cases, dsts, sizes))
           if d[:sz].cpu().numpy().tobytes() != oracle.compress(recipe, arr, w).tobytes()]
    assert not bad, bad[:10]
