#!/usr/bin/env python3
"""Throughput benchmark of the GPU decode path on the mixed-frame workload.

Workload ("mixed_frames_4096"): 4096 independent frames whose sizes are
log-uniform in 4 KiB..4 MiB, element width uniform over {1, 2, 4, 8} bytes,
values a random walk with a per-frame step width log-uniform in [1, 2^16]
(steps uniform in [-s, s], wrapping at the element width). Each frame uses,
by seed, delta -> transpose-split -> FSE or delta -> bitpack_int -> Huffman,
format version 23 with both checksums. Inputs are generated on the host
(numpy, seeded), compressed on the device by the batched encoder, and the
frames are planned once for batched decode.

Timed step (`value`): one CUDA-graph launch decoding all 4096 frames from
HBM into HBM, device-side checksum verification included. The decoded
working set (~2.3 GiB) is larger than L2, so no flush is needed between
steps. `e2e`: the same through ozl_gpu_batch_run_host with pinned host
buffers (frames in, decoded bytes out, copies inside the timed region).
`plain`: the same frames decoded one frame per call through
ozl_gpu_decompress (host planning, stage-by-stage launches, one frame at a
time). `cpu_baseline`: the CPU decoder (the reference's own library where it
runs on this host, else the C restatement in oracle/) over the same frames.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "decompressed GB/s on 1 GB300 (bit-exact): batched vs plain, %HBM peak; p99 ms"
WORKLOAD = "mixed_frames_4096"
RECIPE_TSPLIT_FSE = 3   # delta -> to-struct -> transpose-split(FSE)
RECIPE_BITPACK_HUF = 4  # delta -> bitpack_int -> Huffman
RECIPE_DZ_BITPACK_HUF = 2  # delta -> zigzag -> bitpack_int -> Huffman
OUT_ALIGN = 256
FRAME_ALIGN = 16
# where the CPU baseline is the C restatement (a host that cannot build the
# reference), what it stands for
PORT_NOTE = ("C restatement of the reference's decoder/encoder (oracle/); the reference's own library is "
             "not buildable on this host")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--frames", type=int, default=4096)
    p.add_argument("--seed", type=int, default=20261203)
    p.add_argument("--cpu-threads", type=int, default=0, help="0 = all host cores")
    p.add_argument("--parts-per-kind", type=int, default=None,
                   help="batch decode: runs of frames per kind decoded as parallel graph branches (default: library's)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-plain", action="store_true", help="skip the per-frame plain path")
    p.add_argument("--no-serve", action="store_true", help="skip the serving-loop run")
    p.add_argument("--no-single", action="store_true", help="skip the single 256 MiB array run")
    p.add_argument("--no-columnar", action="store_true", help="skip the columnar/bf16 round trip")
    p.add_argument("--serve-rates", default="1000,2000,5000,10000,20000,50000",
                   help="request rates (req/s) for the serving run")
    p.add_argument("--serve-seconds", type=float, default=1.0, help="seconds of arrivals per rate")
    p.add_argument("--serve-workers", type=int, default=4, help="serving loop worker threads (one stream each)")
    p.add_argument("--serve-requests", type=int, default=0,
                   help="requests per rate (0: --serve-seconds of arrivals per rate)")
    p.add_argument("--no-parity", action="store_true", help="skip the encode-parity check against the oracle")
    p.add_argument("--fse-kernel", type=int, default=None,
                   help="batch decode: FSE kernel (1 a lane per stream, 2 a lane per state); skips the autotuner")
    p.add_argument("--critical-symbols", type=int, default=None,
                   help="batch decode: frames with an FSE stream of at least this many symbols as their own "
                        "branch (0 off; default: the library's, by batch size)")
    p.add_argument("--schedule", type=int, default=None,
                   help="batch decode: branch priorities (0 by branch rank, 1 element-wise launches first)")
    return p.parse_args()


# ---------------------------------------------------------------------------
# workload


def workload_spec(seed, nframes):
    rng = np.random.default_rng(seed)
    size = np.exp(rng.uniform(np.log(4096), np.log(4 << 20), nframes)).astype(np.int64)
    width = rng.choice(np.array([1, 2, 4, 8]), nframes)
    step = np.exp(rng.uniform(0.0, np.log(65536.0), nframes)).astype(np.int64)
    recipe = np.where(rng.random(nframes) < 0.5, RECIPE_TSPLIT_FSE, RECIPE_BITPACK_HUF)
    start = rng.integers(0, 1 << 40, nframes)
    fseed = rng.integers(0, 1 << 62, nframes)
    n = np.maximum(size // width, 1)
    return [dict(n=int(n[i]), w=int(width[i]), step=int(step[i]), recipe=int(recipe[i]), start=int(start[i]),
                 seed=int(fseed[i])) for i in range(nframes)]


_UDT = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def make_frame_input(f, out=None):
    """The frame's little-endian elements as uint8 (written into `out` if given)."""
    rng = np.random.default_rng(f["seed"])
    s = f["step"]
    v = np.cumsum(rng.integers(-s, s + 1, f["n"], dtype=np.int64))
    v += f["start"]
    a = v.astype(_UDT[f["w"]]).view(np.uint8)
    if out is not None:
        out[:a.size] = a
        return out[:a.size]
    return a


def workload_config(n_frames, decoded, compressed, parts_per_kind):
    """The `config` object of both arms' lines (same workload, same frames)."""
    return {"workload": WORKLOAD, "frames": n_frames, "decoded_bytes": decoded, "compressed_bytes": compressed,
            "ratio": round(decoded / compressed, 3), "graphs": "delta->tsplit->FSE | delta->bitpack->Huffman",
            "format_version": 23, "checksums": "content+compressed, verified on decode",
            "l2": "inputs larger than L2 (no flush)", "parts_per_kind": parts_per_kind or "library default",
            "branches": "parallel branches at falling stream priorities: frames with an FSE stream of 16,000+ "
                        "symbols, then runs of the Huffman frames and of the others (library default for batches "
                        "of 512 MiB or more)"}


def layout(sizes, align):
    offs, pos = [], 0
    for s in sizes:
        offs.append(pos)
        pos += (int(s) + align - 1) // align * align
    return offs, max(pos, align)


def host_threads(requested):
    if requested > 0:
        return requested
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# CPU decoders (the reference library where it loads, else the oracle port)


class CpuDecoder:
    def __init__(self):
        self.kind = "port"
        self._ref = None
        ref = os.path.join(ROOT, "oracle", "_ref", "ref_driver.so")
        if os.path.exists(ref):
            try:
                l = ctypes.CDLL(ref)
                l.ref_decompress_into.restype = ctypes.c_int64
                l.ref_decompress_into.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                                  ctypes.c_size_t, ctypes.c_int]
                self._ref = l
                self.kind = "reference"
            except OSError:
                self._ref = None
        if self._ref is None:
            from oracle import oracle

            self._port = oracle.lib()

    def decode(self, src_ptr, src_size, dst_ptr, dst_cap):
        if self._ref is not None:
            return self._ref.ref_decompress_into(src_ptr, src_size, dst_ptr, dst_cap, 1)
        t, w = ctypes.c_int(), ctypes.c_int()
        return self._port.ozo_decompress(src_ptr, src_size, dst_ptr, dst_cap, ctypes.byref(t), ctypes.byref(w))


class CpuEncoder:
    """The CPU compressor of the same graphs: the reference library where it
    loads on this host, else the C restatement in oracle/."""

    def __init__(self):
        self.kind = "port"
        self._ref = None
        ref = os.path.join(ROOT, "oracle", "_ref", "ref_driver.so")
        if os.path.exists(ref):
            try:
                l = ctypes.CDLL(ref)
                l.ref_compress.restype = ctypes.c_int64
                l.ref_compress.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
                self._ref = l
                self.kind = "reference"
            except OSError:
                self._ref = None
        if self._ref is None:
            from oracle import oracle

            self._port = oracle.lib()

    def encode(self, recipe, src_ptr, nb_elts, width, dst_ptr, dst_cap):
        if self._ref is not None:
            return self._ref.ref_compress(recipe, src_ptr, nb_elts, width, dst_ptr, dst_cap, 1, 0)
        return self._port.ozo_compress(recipe, src_ptr, nb_elts, width, dst_ptr, dst_cap, 1)


def cpu_encode_rate(spec, host_in, ooffs, osizes, idx, threads, min_seconds=2.0):
    """CPU compression of frames `idx` on `threads` host threads, repeated
    for at least min_seconds. Returns (GB/s of input bytes, passes)."""
    enc = CpuEncoder()
    caps = [2 * osizes[i] + 4096 for i in idx]
    bufs = [np.empty(c, np.uint8) for c in caps]
    base = host_in.ctypes.data

    def one(k):
        i = idx[k]
        f = spec[i]
        r = enc.encode(f["recipe"], base + ooffs[i], f["n"], f["w"], bufs[k].ctypes.data, caps[k])
        if r <= 0:
            raise RuntimeError("CPU encode of frame %d failed (%d)" % (i, r))
        return osizes[i]

    secs, nb, reps = 0.0, 0, 0
    while reps < 2 or secs < min_seconds:
        t0 = time.perf_counter()
        if threads == 1:
            nb += sum(one(k) for k in range(len(idx)))
        else:
            with ThreadPoolExecutor(threads) as ex:
                nb += sum(ex.map(one, range(len(idx)), chunksize=2))
        secs += time.perf_counter() - t0
        reps += 1
        if reps >= 10:
            break
    return nb / secs / 1e9, reps, enc.kind


def cpu_decode_pass(dec, frames_h, foffs, fsizes, out_h, ooffs, osizes, idx, threads):
    """Decodes frames `idx` on `threads` host threads (ctypes drops the GIL).
    Returns (seconds, decoded bytes)."""
    fbase = frames_h.ctypes.data
    obase = out_h.ctypes.data

    def one(i):
        r = dec.decode(fbase + foffs[i], fsizes[i], obase + ooffs[i], osizes[i])
        if r != osizes[i]:
            raise RuntimeError("CPU decode of frame %d failed (%d)" % (i, r))
        return r

    t0 = time.perf_counter()
    if threads == 1:
        total = sum(one(i) for i in idx)
    else:
        with ThreadPoolExecutor(threads) as ex:
            total = sum(ex.map(one, idx, chunksize=4))
    return time.perf_counter() - t0, total


def cpu_sample(spec, osizes, budget_bytes, seed):
    order = np.random.default_rng(seed + 7).permutation(len(spec))
    idx, tot = [], 0
    for i in order:
        idx.append(int(i))
        tot += osizes[i]
        if tot >= budget_bytes:
            break
    return idx


# ---------------------------------------------------------------------------
# clocks sampled during the timed region


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=5)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = max(smax, float(p[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic_per_algo_byte(name="fse_decode_mixed_frames.md"):
    """DRAM bytes per algorithmic byte of a kernel, from its committed ncu
    summary under profiles/ (line 'dram_bytes_per_algorithmic_byte: X'), or
    None."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("dram_bytes_per_algorithmic_byte:"):
                    return float(line.split(":", 1)[1])
    except (OSError, ValueError):
        pass
    return None


# committed ncu summaries that state a DRAM-bytes-per-algorithmic-byte ratio,
# by (workload, kernel kind)
TRAFFIC_PROFILES = {
    ("mixed_frames_4096", "fse"): "fse_decode_mixed_frames.md",
    ("timestamps_int64_256mib", "huffman"): "huf_decode_timestamps.md",
    ("mixed_frames_4096", "huffman"): "huf_decode_mixed_frames.md",
}


def roofline_from_profile(prof, step_ms, algo_bytes, peak, peak_src, workload):
    """Roofline of the dominant launch kind of one planned run, from its
    per-launch profile [(kind, ms, algorithmic bytes)], with the whole-step
    figures beside it."""
    by_kind = {}
    for kind, ms, nb in prof:
        e = by_kind.setdefault(kind, [0.0, 0, 0])
        e[0] += ms
        e[1] += nb
        e[2] += 1
    prof_ms = sum(v[0] for v in by_kind.values())
    top = max(by_kind, key=lambda k: by_kind[k][0])
    top_ms, top_bytes, top_n = by_kind[top]
    achieved = top_bytes / top_n / (top_ms / top_n / 1e3) / 1e9
    prof_name = TRAFFIC_PROFILES.get((workload, top))
    tpa = ncu_traffic_per_algo_byte(prof_name) if prof_name else None
    return {
        "bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4), "peak_source": peak_src,
        "traffic": round(tpa * top_bytes / top_n) if tpa else None,
        "algorithmic_bytes_per_launch": int(top_bytes / top_n), "launches": top_n,
        "share_of_step": round(top_ms / prof_ms, 4),
        "step": {"achieved": round(algo_bytes / (step_ms / 1e3) / 1e9, 1),
                 "frac": round(algo_bytes / (step_ms / 1e3) / 1e9 / peak, 4),
                 "algorithmic_bytes": int(algo_bytes)},
        "kinds": {k: {"ms": round(v[0], 4), "launches": v[2], "gbs": round(v[1] / (v[0] / 1e3) / 1e9, 1)}
                  for k, v in sorted(by_kind.items(), key=lambda kv: -kv[1][0])},
        "per_launch": [[kind, round(ms, 4), int(nb)] for kind, ms, nb in prof],
    }


def timed_batch_runs(torch, batch, stream, sptr, reps):
    """Milliseconds per graph launch of a planned batch, CUDA events on the
    launching stream over `reps` launches."""
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        batch.run(sptr, graph=True)
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def encode_parity(pairs, threads):
    """GPU frames against the CPU restatement's frames for the same inputs
    and graphs (the restatement is pinned byte for byte to the reference's
    frames by the test suite). pairs: [(label, recipe, host array, elt width,
    GPU frame as uint8)]. Returns {label: [checked, equal]}."""
    from oracle import oracle

    def one(p):
        label, r, a, w, fr = p
        want = oracle.compress(r, a, w, checksums=True)
        return label, bool(want.size == fr.size and np.array_equal(want, fr))

    out = {}
    with ThreadPoolExecutor(threads) as ex:
        for label, eq in ex.map(one, pairs):
            e = out.setdefault(label, [0, 0])
            e[0] += 1
            e[1] += int(eq)
    return out


# ---------------------------------------------------------------------------
# distributed helpers (one process per GPU; frames shard by rank)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def build_workload_host(spec, threads):
    """Inputs laid out back to back (OUT_ALIGN) in one host array."""
    osizes = [f["n"] * f["w"] for f in spec]
    ooffs, obytes = layout(osizes, OUT_ALIGN)
    host_in = np.zeros(obytes, np.uint8)

    def gen(i):
        make_frame_input(spec[i], host_in[ooffs[i]:ooffs[i] + osizes[i]])

    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(gen, range(len(spec)), chunksize=8))
    return host_in, ooffs, osizes, obytes


# ---------------------------------------------------------------------------
# single large array (256 MiB int64 timestamps, delta -> zigzag -> bitpack ->
# Huffman), decoded by the plain per-frame path


def timestamps(seed, n):
    rng = np.random.default_rng(seed)
    inc = rng.geometric(1 / 1000, n).astype(np.int64)
    out = rng.random(n) < 0.01
    inc[out] = rng.integers(0, 1 << 32, int(out.sum()))
    return (1700000000000000000 + np.cumsum(inc)).astype(np.int64)


def run_single_array(oz, torch, dev, stream, sptr, seed, peak, peak_src, parity):
    """The 256 MiB timestamp array: GPU encode, the plain per-frame decode
    (host plan plus stage-by-stage launches per call), the same frame as a
    one-frame captured graph (CUDA events, per-launch roofline), and the CPU
    decoder on the same frame on one core."""
    n = 256 << 17  # 33,554,432 int64 values = 256 MiB
    a = timestamps(seed + 2, n)
    d_in = torch.from_numpy(a.view(np.uint8)).to(dev)
    enc = oz.GpuEncoder()
    cap = enc.bound(a.nbytes)
    d_fr = torch.empty(cap, dtype=torch.uint8, device=dev)
    fs = enc.compress_batch([d_in.data_ptr()], [n], [8], [RECIPE_DZ_BITPACK_HUF], [d_fr.data_ptr()], [cap],
                            checksums=True, stream=sptr)[0]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    enc.compress_batch([d_in.data_ptr()], [n], [8], [RECIPE_DZ_BITPACK_HUF], [d_fr.data_ptr()], [cap],
                       checksums=True, stream=sptr)
    torch.cuda.synchronize()
    enc_s = time.perf_counter() - t0
    frame_h = d_fr[:fs].cpu().numpy()
    parity.append(("timestamps_int64_256mib", RECIPE_DZ_BITPACK_HUF, a, 8, frame_h))
    d_out = torch.empty(a.nbytes, dtype=torch.uint8, device=dev)
    dctx = oz.DCtx()
    for _ in range(2):
        dctx.decompress_device(frame_h, d_fr.data_ptr(), d_out.data_ptr(), a.nbytes, stream=sptr)
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        dctx.decompress_device(frame_h, d_fr.data_ptr(), d_out.data_ptr(), a.nbytes, stream=sptr)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    if not torch.equal(d_out, d_in):
        raise RuntimeError("single-array decode differs from the input")
    # the same frame as a captured one-frame graph
    batch = oz.GpuBatch()
    batch.plan([frame_h], [d_fr.data_ptr()], [d_out.data_ptr()], [a.nbytes])
    d_out.zero_()
    torch.cuda.nvtx.range_push("single")  # a profiler can select these launches
    for _ in range(3):
        batch.run(sptr, graph=True)
    torch.cuda.nvtx.range_pop()
    batch.check(sptr)
    graph_ms = timed_batch_runs(torch, batch, stream, sptr, 10)
    batch.check(sptr)
    if not torch.equal(d_out, d_in):
        raise RuntimeError("single-array graph decode differs from the input")
    roof = roofline_from_profile(batch.profile(sptr, capacity=64), graph_ms, a.nbytes + fs, peak, peak_src,
                                 "timestamps_int64_256mib")
    # CPU decoder on the same frame (one frame: one core, as in the reference)
    dec = CpuDecoder()
    out_c = np.empty(a.nbytes, np.uint8)
    fr_c = np.ascontiguousarray(frame_h)
    times = []
    for _ in range(2):
        t1 = time.perf_counter()
        r = dec.decode(fr_c.ctypes.data, fs, out_c.ctypes.data, a.nbytes)
        times.append(time.perf_counter() - t1)
        if r != a.nbytes:
            raise RuntimeError("CPU decode of the single array failed (%d)" % r)
    if not np.array_equal(out_c, a.view(np.uint8)):
        raise RuntimeError("CPU decode of the single array differs")
    cpu = {"value": round(a.nbytes / min(times) / 1e9, 4), "unit": "GB/s", "cores": 1, "kind": dec.kind,
           "sample": "the whole 256 MiB frame, 1 thread, best of 2"}
    return {"workload": "timestamps_int64_256mib", "graph": "delta->zigzag->bitpack->Huffman",
            "decoded_bytes": int(a.nbytes), "compressed_bytes": int(fs), "ratio": round(a.nbytes / fs, 3),
            "plain_gbs": round(a.nbytes / dt / 1e9, 2), "ms": round(dt * 1e3, 3),
            "graph_gbs": round(a.nbytes / (graph_ms / 1e3) / 1e9, 2), "graph_ms": round(graph_ms, 3),
            "encode_gbs": round(a.nbytes / enc_s / 1e9, 2), "roofline": roof, "cpu_baseline": cpu}


# ---------------------------------------------------------------------------
# columnar and weight-like data: a 64M-row int32 column (Zipf 1.1 over 10,000
# random keys) through tokenize -> {alphabet: store, indices: bitpack ->
# Huffman}, and 2 GiB of bf16 matrices (4096x4096, 4096x11008, 11008x4096,
# N(0, 0.02)) through bf16 deconstruct -> {sign|fraction: store, exponent:
# FSE}; all frames encoded in one batched call and decoded in one batched
# graph launch, checked bit-exact


RECIPE_TOKENIZE = 5
RECIPE_BF16 = 6


def run_columnar(oz, torch, dev, stream, sptr, seed, peak, peak_src, threads, parity):
    g = torch.Generator(device=dev)
    g.manual_seed(seed + 41)
    rows = 64 << 20
    keys = torch.randint(0, 2**31 - 1, (10000,), device=dev, generator=g, dtype=torch.int64).to(torch.int32)
    p = 1.0 / torch.arange(1, 10001, device=dev, dtype=torch.float64) ** 1.1
    cdf = torch.cumsum(p / p.sum(), 0)
    u = torch.rand(rows, device=dev, generator=g, dtype=torch.float64)
    col = keys[torch.searchsorted(cdf, u).clamp_(max=9999)].contiguous()
    shapes = [(4096, 4096), (4096, 11008), (11008, 4096)] * 10
    mats = [(torch.randn(r, c, device=dev, generator=g) * 0.02).to(torch.bfloat16).contiguous() for r, c in shapes]
    srcs = [col] + mats
    nbytes = [t.numel() * t.element_size() for t in srcs]
    elts = [t.numel() for t in srcs]
    widths = [4] + [2] * len(mats)
    recipes = [RECIPE_TOKENIZE] + [RECIPE_BF16] * len(mats)
    enc = oz.GpuEncoder()
    caps = [enc.bound(b) for b in nbytes]
    offs, tot = layout(caps, OUT_ALIGN)
    d_fr = torch.empty(tot, dtype=torch.uint8, device=dev)
    fptr = [d_fr.data_ptr() + o for o in offs]
    enc.compress_batch([t.data_ptr() for t in srcs], elts, widths, recipes, fptr, caps, checksums=True, stream=sptr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fs = enc.compress_batch([t.data_ptr() for t in srcs], elts, widths, recipes, fptr, caps, checksums=True,
                            stream=sptr)
    torch.cuda.synchronize()
    enc_s = time.perf_counter() - t0
    frames_h = [d_fr[o:o + f].cpu().numpy() for o, f in zip(offs, fs)]
    # encode parity: the column and one matrix of each shape
    host_src = {}
    for k in (0, 1, 2, 3):
        h = srcs[k].view(torch.uint8).reshape(-1).cpu().numpy()
        host_src[k] = h
        arr = h.view(np.uint32) if k == 0 else h.view(np.uint16)
        parity.append(("columnar_zipf_int32" if k == 0 else "bf16_weights", recipes[k], arr, widths[k], frames_h[k]))
    ooffs, obytes = layout(nbytes, OUT_ALIGN)
    d_out = torch.zeros(obytes, dtype=torch.uint8, device=dev)
    batch = oz.GpuBatch()
    batch.plan(frames_h, fptr, [d_out.data_ptr() + o for o in ooffs], nbytes)
    for _ in range(3):
        batch.run(sptr, graph=True)
    batch.check(sptr)
    dec_ms = timed_batch_runs(torch, batch, stream, sptr, 10)
    batch.check(sptr)
    ok = all(torch.equal(d_out[o:o + n], t.view(torch.uint8).reshape(-1)) for o, n, t in zip(ooffs, nbytes, srcs))
    if not ok:
        raise RuntimeError("columnar round trip differs")
    total = sum(nbytes)
    roof = roofline_from_profile(batch.profile(sptr, capacity=256), dec_ms, total + sum(fs), peak, peak_src,
                                 "columnar_bf16")
    # CPU decoder: the column and the first six matrices, all host threads
    dec = CpuDecoder()
    sel = list(range(7))
    fr_c = [np.ascontiguousarray(frames_h[k]) for k in sel]
    out_c = [np.empty(nbytes[k], np.uint8) for k in sel]

    def one(j):
        k = sel[j]
        r = dec.decode(fr_c[j].ctypes.data, fs[k], out_c[j].ctypes.data, nbytes[k])
        if r != nbytes[k]:
            raise RuntimeError("CPU decode of columnar frame %d failed (%d)" % (k, r))
        return r

    cpu_times = []
    for _ in range(2):
        t1 = time.perf_counter()
        with ThreadPoolExecutor(min(threads, len(sel))) as ex:
            cpu_bytes = sum(ex.map(one, range(len(sel))))
        cpu_times.append(time.perf_counter() - t1)
    for j, k in enumerate(sel[:4]):
        if k in host_src and not np.array_equal(out_c[j], host_src[k]):
            raise RuntimeError("CPU decode of columnar frame %d differs" % k)
    cpu = {"value": round(cpu_bytes / min(cpu_times) / 1e9, 4), "unit": "GB/s", "cores": min(threads, len(sel)),
           "kind": dec.kind, "sample": "the column and 6 of the 30 matrices (%.0f MiB), one frame per thread, best of 2"
           % (cpu_bytes / 2**20)}
    return {"column_rows": rows, "column_ratio": round(nbytes[0] / fs[0], 3), "bf16_bytes": sum(nbytes[1:]),
            "bf16_ratio": round(sum(nbytes[1:]) / sum(fs[1:]), 3), "frames": len(srcs),
            "encode_gbs": round(total / enc_s / 1e9, 2), "decode_gbs": round(total / (dec_ms / 1e3) / 1e9, 2),
            "decode_ms": round(dec_ms, 3), "bit_exact": True, "roofline": roof, "cpu_baseline": cpu}


# ---------------------------------------------------------------------------
# serving loop: Poisson arrivals of decompress (80 %) and compress (20 %)
# requests, payloads log-normal (median 256 KiB, sigma 1.5, clipped to
# 1 KiB..64 MiB) from the timestamp and random-walk generators


def serving_pool(seed, count):
    rng = np.random.default_rng(seed + 11)
    sizes = np.clip(np.exp(rng.normal(np.log(256 << 10), 1.5, count)), 1 << 10, 64 << 20).astype(np.int64)
    pool = []
    for i, b in enumerate(sizes):
        if i % 2 == 0:
            a = timestamps(seed + 100 + i, max(int(b) // 8, 1))
            pool.append((a.view(np.uint8), 8, RECIPE_DZ_BITPACK_HUF))
        else:
            w = int(rng.choice([1, 2, 4, 8]))
            f = dict(n=max(int(b) // w, 1), w=w, step=int(np.exp(rng.uniform(0, np.log(65536)))),
                     recipe=int(rng.choice([RECIPE_TSPLIT_FSE, RECIPE_BITPACK_HUF])),
                     start=int(rng.integers(0, 1 << 40)), seed=int(rng.integers(0, 1 << 62)))
            pool.append((make_frame_input(f), w, f["recipe"]))
    return pool


def run_serving(oz, torch, dev, sptr, args):
    pool = serving_pool(args.seed, 96)
    enc = oz.GpuEncoder()
    # frames of every pool entry, compressed on the device
    d_in = [torch.from_numpy(p[0].copy()).to(dev) for p in pool]
    caps = [enc.bound(p[0].nbytes) for p in pool]
    d_fr = [torch.empty(c, dtype=torch.uint8, device=dev) for c in caps]
    fs = enc.compress_batch([d.data_ptr() for d in d_in], [p[0].nbytes // p[1] for p in pool], [p[1] for p in pool],
                            [p[2] for p in pool], [d.data_ptr() for d in d_fr], caps, checksums=True, stream=sptr)
    torch.cuda.synchronize()
    frames = [d_fr[i][:fs[i]].cpu().numpy() for i in range(len(pool))]
    del d_in, d_fr

    def pinned(nbytes):
        return torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True).numpy()

    frames_p, src_p = [], []
    for i, p in enumerate(pool):
        f = pinned(frames[i].size)
        f[:frames[i].size] = frames[i]
        frames_p.append(f[:frames[i].size])
        x = pinned(p[0].nbytes)
        x[:p[0].nbytes] = p[0]
        src_p.append(x[:p[0].nbytes])
    slots = 4
    outs_d = [[pinned(p[0].nbytes) for _ in range(slots)] for p in pool]
    outs_c = [[pinned(caps[i]) for _ in range(slots)] for i in range(len(pool))]
    rng = np.random.default_rng(args.seed + 5)
    srv = oz.Server(hbm_budget=40 << 30, workers=args.serve_workers, checksums=True)
    results = []
    rates = [int(r) for r in args.serve_rates.split(",") if r]
    for rate in rates:
        nreq = args.serve_requests if args.serve_requests > 0 else max(50, int(rate * args.serve_seconds))
        gaps = rng.exponential(1.0 / rate, nreq)
        kinds = rng.random(nreq) < 0.8
        which = rng.integers(0, len(pool), nreq)
        lat, nbytes, done = [], 0, 0
        st0 = srv.stats()
        t0 = time.perf_counter()
        due = t0
        last_poll = t0
        for k in range(nreq):
            due += gaps[k]
            while True:  # wait for the arrival time, draining completions every 0.2 ms
                now = time.perf_counter()
                if now - last_poll > 2e-4:
                    for _, code, val, lus in srv.poll(wait_ms=0):
                        if code:
                            raise RuntimeError("serving request failed (%d)" % code)
                        lat.append(lus)
                        done += 1
                    last_poll = now
                if now >= due:
                    break
            i = int(which[k])
            if kinds[k]:
                srv.submit_decompress(frames_p[i], outs_d[i][k % slots])
            else:
                srv.submit_compress(src_p[i], pool[i][1], pool[i][2], outs_c[i][k % slots])
            nbytes += pool[i][0].nbytes
        while done < nreq:
            for _, code, val, lus in srv.poll(wait_ms=50):
                if code:
                    raise RuntimeError("serving request failed (%d)" % code)
                lat.append(lus)
                done += 1
        wall = time.perf_counter() - t0
        lat = np.sort(np.array(lat)) / 1e3
        st1 = srv.stats()
        results.append({"rate": rate, "requests": nreq, "p50_ms": round(float(np.percentile(lat, 50)), 3),
                        "p99_ms": round(float(np.percentile(lat, 99)), 3), "gbs": round(nbytes / wall / 1e9, 2),
                        "offered_gbs": round(nbytes / (gaps.sum()) / 1e9, 2),
                        "workers_s": {k: round(st1[k] - st0[k], 4) for k in st1}, "wall_s": round(wall, 4)})
    srv.close()
    # plain per-request path: the same kind of requests one call at a time
    # through the reference-style API (ZL_DCtx_decompressTyped /
    # ZL_CCtx_compressTypedRef with host buffers)
    d = oz.DCtx()
    comps = {}
    for r in (RECIPE_TSPLIT_FSE, RECIPE_BITPACK_HUF, RECIPE_DZ_BITPACK_HUF):
        c = oz.Compressor()
        a = oz.api
        if r == RECIPE_TSPLIT_FSE:
            g = c.pipeline([a.NODE_DELTA_INT, a.NODE_CONVERT_NUM_TO_TOKEN], c.transpose_split(a.GRAPH_FSE))
        elif r == RECIPE_BITPACK_HUF:
            g = c.node(a.NODE_DELTA_INT, c.node(a.NODE_BITPACK_INT, a.GRAPH_HUFFMAN))
        else:
            g = c.pipeline([a.NODE_DELTA_INT, a.NODE_ZIGZAG], c.node(a.NODE_BITPACK_INT, a.GRAPH_HUFFMAN))
        c.select(g)
        cc = oz.CCtx()
        cc.ref_compressor(c)
        cc.set_parameter(a.CPARAM_STICKY, 1)
        cc.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
        comps[r] = (c, cc)
    npl = 300
    kinds = rng.random(npl) < 0.8
    which = rng.integers(0, len(pool), npl)
    nbytes = 0
    t0 = time.perf_counter()
    for k in range(npl):
        i = int(which[k])
        if kinds[k]:
            d.decompress_typed(frames_p[i], outs_d[i][0])
        else:
            _, w, r = pool[i]
            comps[r][1].compress_numeric(src_p[i].view({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[w]))
        nbytes += pool[i][0].nbytes
    plain_gbs = nbytes / (time.perf_counter() - t0) / 1e9
    return {"workers": args.serve_workers, "hbm_budget_gb": 40, "mix": "80% decompress / 20% compress",
            "payload": "log-normal, median 256 KiB, sigma 1.5, clipped 1 KiB..64 MiB", "pool": len(pool),
            "host_buffers": "pinned", "rates": results, "plain_per_request_gbs": round(plain_gbs, 3)}


# ---------------------------------------------------------------------------
# reference arm: the CPU decoder over the same workload


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle

    threads = host_threads(args.cpu_threads)
    spec = workload_spec(args.seed, args.frames)
    host_in, ooffs, osizes, obytes = build_workload_host(spec, threads)
    # frames from the CPU encoder of the same graphs (identical to the GPU's)
    frames = [None] * len(spec)

    def enc(i):
        f = spec[i]
        a = host_in[ooffs[i]:ooffs[i] + osizes[i]].view(_UDT[f["w"]])
        frames[i] = oracle.compress(f["recipe"], a, f["w"], checksums=True)

    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(enc, range(len(spec)), chunksize=4))
    fsizes = [fr.size for fr in frames]
    foffs, fbytes = layout(fsizes, FRAME_ALIGN)
    frames_h = np.zeros(fbytes, np.uint8)
    for i, fr in enumerate(frames):
        frames_h[foffs[i]:foffs[i] + fsizes[i]] = fr
    out_h = np.zeros(obytes, np.uint8)
    dec = CpuDecoder()
    # each step decodes the whole workload (every frame), as our arm does
    idx = list(range(len(spec)))
    for _ in range(args.warmup):
        cpu_decode_pass(dec, frames_h, foffs, fsizes, out_h, ooffs, osizes, idx, threads)
    times, nbytes = [], 0
    for _ in range(args.steps):
        t, b = cpu_decode_pass(dec, frames_h, foffs, fsizes, out_h, ooffs, osizes, idx, threads)
        times.append(t)
        nbytes = b
    for i in idx:
        if not np.array_equal(out_h[ooffs[i]:ooffs[i] + osizes[i]], host_in[ooffs[i]:ooffs[i] + osizes[i]]):
            raise RuntimeError("CPU decode mismatch on frame %d" % i)
    tot = sum(times)
    gbs = nbytes * len(times) / tot / 1e9
    sample = "%d of %d frames (%.1f MiB decoded per step), %d threads" % (len(idx), len(spec), nbytes / 2**20,
                                                                          threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 4), "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot / len(times) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded random walks)",
        "config": workload_config(len(spec), int(sum(osizes)), int(sum(fsizes)), args.parts_per_kind),
        "cpu_baseline": {"value": round(gbs, 4), "unit": "GB/s", "cores": threads, "kind": dec.kind,
                         "sample": sample, **({"note": PORT_NOTE} if dec.kind == "port" else {})},
        "e2e": {"value": round(gbs, 4), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)

    import torch

    ws, rank, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import openzl_gb300 as oz

    threads = host_threads(args.cpu_threads)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream

    # ---- inputs (frames shard by rank: each rank codes its own seeded set)
    spec = workload_spec(args.seed + 7919 * rank, args.frames)
    host_in, ooffs, osizes, obytes = build_workload_host(spec, threads)
    n_frames = len(spec)
    total_out = int(sum(osizes))
    d_in = torch.from_numpy(host_in).to(dev)

    # ---- compress on the device (batched encoder)
    enc = oz.GpuEncoder()
    bounds = [enc.bound(s) for s in osizes]
    boffs, bbytes = layout(bounds, OUT_ALIGN)
    d_slots = torch.empty(bbytes, dtype=torch.uint8, device=dev)
    in_ptrs = [d_in.data_ptr() + o for o in ooffs]
    slot_ptrs = [d_slots.data_ptr() + o for o in boffs]
    nb_elts = [f["n"] for f in spec]
    widths = [f["w"] for f in spec]
    recipes = [f["recipe"] for f in spec]
    with torch.cuda.stream(stream):
        torch.cuda.synchronize()
        fsizes = enc.compress_batch(in_ptrs, nb_elts, widths, recipes, slot_ptrs, bounds, checksums=True,
                                    stream=sptr)
        enc_times = []
        # NVTX range: a profiler can pick the timed encode calls
        # (ncu --nvtx --nvtx-include "encode/")
        torch.cuda.nvtx.range_push("encode")
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            enc.compress_batch(in_ptrs, nb_elts, widths, recipes, slot_ptrs, bounds, checksums=True, stream=sptr)
            torch.cuda.synchronize()
            enc_times.append(time.perf_counter() - t0)
        torch.cuda.nvtx.range_pop()
    enc_gbs = total_out / min(enc_times) / 1e9
    enc_phases = enc.phases()  # of the last timed call
    enc_launches = enc.launches() if hasattr(enc, "launches") else None

    # compact the frames back to back (FRAME_ALIGN) for the host-buffer path
    foffs, fbytes = layout(fsizes, FRAME_ALIGN)
    d_frames = torch.zeros(fbytes, dtype=torch.uint8, device=dev)
    for i in range(n_frames):
        d_frames[foffs[i]:foffs[i] + fsizes[i]].copy_(d_slots[boffs[i]:boffs[i] + fsizes[i]])
    del d_slots
    frames_h = torch.empty(fbytes, dtype=torch.uint8, pin_memory=True)
    frames_h.copy_(d_frames)
    frames_np = frames_h.numpy()
    total_comp = int(sum(fsizes))

    # ---- plan the batched decode
    d_out = torch.zeros(obytes, dtype=torch.uint8, device=dev)
    batch = oz.GpuBatch(parts_per_kind=args.parts_per_kind, fse_kernel=args.fse_kernel,
                        critical_symbols=args.critical_symbols, schedule=args.schedule)
    host_views = [frames_np[foffs[i]:foffs[i] + fsizes[i]] for i in range(n_frames)]
    planned = batch.plan(host_views, [d_frames.data_ptr() + o for o in foffs],
                         [d_out.data_ptr() + o for o in ooffs], osizes)
    assert planned == total_out, (planned, total_out)

    # autotuner: launch shapes (chunks per CTA of the FSE and Huffman launches)
    prof0 = sum(ms for _, ms, _ in batch.profile(sptr, capacity=256))
    if args.fse_kernel is None:
        shapes = batch.autotune(sptr, reps=2)
        prof1 = sum(ms for _, ms, _ in batch.profile(sptr, capacity=256))
        tuned = {"shapes": shapes, "profile_ms_before": round(prof0, 3), "profile_ms_after": round(prof1, 3)}
    else:
        tuned = {"fse_kernel": args.fse_kernel, "profile_ms": round(prof0, 3)}

    # warm-up (graph capture happens on the first run); the NVTX range lets a
    # profiler pick the tuned launches (ncu --nvtx --nvtx-include "warmup/")
    torch.cuda.nvtx.range_push("warmup")
    for _ in range(args.warmup):
        batch.run(sptr, graph=True)
    torch.cuda.nvtx.range_pop()
    batch.check(sptr)
    launches = batch.launches()  # kernels in one captured decode step
    if not torch.equal(d_out, d_in):
        raise RuntimeError("batched decode differs from the input")
    d_out.zero_()

    # ---- timed region: K batched decode steps
    clocks = ClockSampler(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    # The K steps queue behind a 0.1 s device-side delay (a bounded clock
    # spin, before the timed region), so that a pause of the host thread
    # (driver queries of the clock sampler have stalled graph launches for
    # milliseconds) cannot open gaps between the steps: the timed region is
    # the device's time for exactly K steps.
    with torch.cuda.stream(stream):
        torch.cuda._sleep(int(0.1 * 2.07e9))
    t_start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        batch.run(sptr, graph=True)
        ev[k][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    total_ms = t_start.elapsed_time(t_end)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    batch.check(sptr)  # device-verified content + compressed checksums of the last step
    if not torch.equal(d_out, d_in):
        raise RuntimeError("batched decode differs from the input after the timed steps")
    ms_per_step = total_ms / args.steps
    value = total_out * ws / (ms_per_step / 1e3) / 1e9

    # ---- roofline: per-launch profile of one run (CUDA events per launch)
    peak, peak_src = measured_hbm_peak()
    prof = batch.profile(sptr, capacity=max(64, launches + 8))
    # concurrency: one run without the graph, an event around every launch on
    # its branch's stream: [branch, kind, level, ms reached, ms ended]
    timeline = [[b_, k_, l_, round(a_, 3), round(e_, 3)] for b_, k_, l_, a_, e_ in batch.timeline(sptr, capacity=256)]
    roofline = roofline_from_profile(prof, ms_per_step, total_out + total_comp, peak, peak_src, WORKLOAD)

    # ---- e2e: host buffers through the C ABI, copies inside the timed region
    out_h = torch.empty(obytes, dtype=torch.uint8, pin_memory=True)
    for _ in range(2):
        batch.run_host(frames_h.data_ptr(), fbytes, out_h.data_ptr(), obytes, sptr, graph=True)
    e2e_steps = max(3, min(args.steps, 10))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.run_host(frames_h.data_ptr(), fbytes, out_h.data_ptr(), obytes, sptr, graph=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if not np.array_equal(out_h.numpy(), host_in):
        raise RuntimeError("host-buffer decode differs from the input")
    e2e = {"value": round(total_out * ws / e2e_s / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": fbytes,
           "d2h_bytes_per_step": obytes, "ms_per_step": round(e2e_s * 1e3, 3)}
    # per round of the host-buffer run: ms its frames were in, decoded, out
    e2e["rounds"] = [[round(a, 3), round(b, 3), round(c, 3)]
                     for a, b, c in batch.host_timeline(frames_h.data_ptr(), fbytes, out_h.data_ptr(), obytes, sptr)]

    # ---- plain path: one frame per call, stage-by-stage launches
    plain = None
    if not args.no_plain:
        dctx = oz.DCtx()
        dptr_f = d_frames.data_ptr()
        dptr_o = d_out.data_ptr()
        for i in range(min(8, n_frames)):
            dctx.decompress_device(host_views[i], dptr_f + foffs[i], dptr_o + ooffs[i], osizes[i], stream=sptr)
        d_out.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(n_frames):
            dctx.decompress_device(host_views[i], dptr_f + foffs[i], dptr_o + ooffs[i], osizes[i], stream=sptr)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - t0
        if not torch.equal(d_out, d_in):
            raise RuntimeError("plain decode differs from the input")
        plain = {"value": round(total_out / plain_s / 1e9, 3), "unit": "GB/s", "ms": round(plain_s * 1e3, 2),
                 "batched_over_plain": round(value / ws / (total_out / plain_s / 1e9), 2)}

    # ---- encode parity: a seeded sample of the mixed frames (GPU frames
    # against the restatement's frames), then the other workloads add theirs
    parity = []
    if rank == 0 and ws == 1 and not args.no_parity:
        for i in cpu_sample(spec, osizes, 1 << 62, args.seed + 3)[:256]:
            f = spec[i]
            a = host_in[ooffs[i]:ooffs[i] + osizes[i]].view(_UDT[f["w"]])
            parity.append((WORKLOAD, f["recipe"], a, f["w"], frames_np[foffs[i]:foffs[i] + fsizes[i]]))

    # ---- the single large array and the serving loop (rank 0, N=1 only)
    single = None
    serving = None
    if rank == 0 and ws == 1 and not args.no_single:
        single = run_single_array(oz, torch, dev, stream, sptr, args.seed, peak, peak_src, parity)
    if rank == 0 and ws == 1 and not args.no_serve:
        serving = run_serving(oz, torch, dev, sptr, args)
    columnar = None
    if rank == 0 and ws == 1 and not args.no_columnar:
        columnar = run_columnar(oz, torch, dev, stream, sptr, args.seed, peak, peak_src, threads, parity)
    enc_parity = None
    if parity:
        t0 = time.perf_counter()
        res = encode_parity(parity, threads)
        enc_parity = {"frames_checked": sum(v[0] for v in res.values()), "equal": sum(v[1] for v in res.values()),
                      "by_workload": {k: {"checked": v[0], "equal": v[1]} for k, v in res.items()},
                      "against": "frames of the CPU restatement, which the test suite pins byte for byte to the "
                                 "reference's frames", "seconds": round(time.perf_counter() - t0, 1)}
        if enc_parity["equal"] != enc_parity["frames_checked"]:
            print("encode parity: %d of %d GPU frames differ from the oracle's" % (
                enc_parity["frames_checked"] - enc_parity["equal"], enc_parity["frames_checked"]), file=sys.stderr)

    # ---- CPU baseline (rank 0, N=1 only): the same frames on the host
    # cores, all threads and one thread; the CPU compressor beside it
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        dec = CpuDecoder()
        idx = cpu_sample(spec, osizes, total_out // 4, args.seed)
        out_c = np.zeros(obytes, np.uint8)

        def decode_rate(sel, nthreads, min_seconds):
            cpu_decode_pass(dec, frames_np, foffs, fsizes, out_c, ooffs, osizes, sel[:16], nthreads)
            reps, secs, nb = 0, 0.0, 0
            while reps < 2 or secs < min_seconds:
                t, b = cpu_decode_pass(dec, frames_np, foffs, fsizes, out_c, ooffs, osizes, sel, nthreads)
                secs += t
                nb += b
                reps += 1
                if reps >= 20:
                    break
            return nb / secs / 1e9, reps

        all_gbs, reps = decode_rate(idx, threads, 3.0)
        for i in idx:
            if not np.array_equal(out_c[ooffs[i]:ooffs[i] + osizes[i]], host_in[ooffs[i]:ooffs[i] + osizes[i]]):
                raise RuntimeError("CPU decode mismatch on frame %d" % i)
        idx1 = cpu_sample(spec, osizes, total_out // 64, args.seed + 1)
        one_gbs, reps1 = decode_rate(idx1, 1, 2.0)
        eidx = cpu_sample(spec, osizes, total_out // 16, args.seed + 2)
        enc_all, _, enc_kind = cpu_encode_rate(spec, host_in, ooffs, osizes, eidx, threads)
        eidx1 = cpu_sample(spec, osizes, total_out // 128, args.seed + 4)
        enc_one, _, _ = cpu_encode_rate(spec, host_in, ooffs, osizes, eidx1, 1)
        cpu = {"value": round(all_gbs, 4), "unit": "GB/s", "cores": threads, "kind": dec.kind,
               "sample": "%d of %d frames (%.1f MiB decoded), %d passes, %d threads" % (
                   len(idx), n_frames, sum(osizes[i] for i in idx) / 2**20, reps, threads),
               "one_core": {"value": round(one_gbs, 4), "unit": "GB/s", "cores": 1,
                            "sample": "%d frames (%.1f MiB), %d passes" % (
                                len(idx1), sum(osizes[i] for i in idx1) / 2**20, reps1)},
               "encode": {"value": round(enc_all, 4), "unit": "GB/s", "cores": threads, "kind": enc_kind,
                          "one_core": round(enc_one, 4),
                          "sample": "%d frames (%.1f MiB) on %d threads; %d frames on 1 thread" % (
                              len(eidx), sum(osizes[i] for i in eidx) / 2**20, threads, len(eidx1))}}
        if dec.kind == "port":
            cpu["note"] = PORT_NOTE

    srt = sorted(step_ms)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded random walks)",
        "config": dict(workload_config(n_frames, total_out, total_comp, args.parts_per_kind),
                       launch="the K timed steps are queued behind a 0.1 s device-side delay before the first event"),
        "frac_hbm": round(value / ws / peak, 4),
        "p50_ms": round(statistics.median(step_ms), 4),
        "p99_ms": round(srt[min(len(srt) - 1, int(round(0.99 * (len(srt) - 1))))], 4),
        "plain": plain,
        "single_array": single,
        "serving": serving,
        "columnar": columnar,
        "encode": {"value": round(enc_gbs, 3), "unit": "GB/s", "note": "batched compress, host decisions included",
                   "phases_ms": enc_phases, "parity": enc_parity},
        "autotune": tuned,
        "timeline": timeline,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "encode_parity": enc_parity,
        "e2e": e2e,
        "gpu_launches": launches * args.steps,
        "clocks": clk,
    }
    if enc_launches is not None:
        line["encode"]["launches"] = enc_launches
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
