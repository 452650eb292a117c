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
OUT_ALIGN = 256
FRAME_ALIGN = 16


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--frames", type=int, default=4096)
    p.add_argument("--seed", type=int, default=20261203)
    p.add_argument("--cpu-threads", type=int, default=0, help="0 = all host cores")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-plain", action="store_true", help="skip the per-frame plain path")
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


def ncu_traffic_per_algo_byte():
    """DRAM bytes per algorithmic byte of the dominant decode kernel, from the
    committed ncu summary (line 'dram_bytes_per_algorithmic_byte: X'), or None."""
    p = os.path.join(ROOT, "profiles", "fse_decode_mixed_frames.md")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("dram_bytes_per_algorithmic_byte:"):
                    return float(line.split(":", 1)[1])
    except (OSError, ValueError):
        pass
    return None


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
    # each step: a bounded sample (1/4 of the workload's bytes)
    idx = cpu_sample(spec, osizes, sum(osizes) // 4, args.seed)
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
        "config": {"workload": WORKLOAD, "frames": len(spec), "decoded_bytes": int(sum(osizes)),
                   "compressed_bytes": int(sum(fsizes)), "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": round(gbs, 4), "unit": "GB/s", "cores": threads, "kind": dec.kind,
                         "sample": sample},
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
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            enc.compress_batch(in_ptrs, nb_elts, widths, recipes, slot_ptrs, bounds, checksums=True, stream=sptr)
            torch.cuda.synchronize()
            enc_times.append(time.perf_counter() - t0)
    enc_gbs = total_out / min(enc_times) / 1e9
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
    batch = oz.GpuBatch()
    host_views = [frames_np[foffs[i]:foffs[i] + fsizes[i]] for i in range(n_frames)]
    planned = batch.plan(host_views, [d_frames.data_ptr() + o for o in foffs],
                         [d_out.data_ptr() + o for o in ooffs], osizes)
    assert planned == total_out, (planned, total_out)

    # warm-up (graph capture happens on the first run)
    for _ in range(args.warmup):
        batch.run(sptr, graph=True)
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
    tpa = ncu_traffic_per_algo_byte()
    roofline = {
        "bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4), "peak_source": peak_src,
        "traffic": round(tpa * top_bytes / top_n) if tpa else None,
        "algorithmic_bytes_per_launch": int(top_bytes / top_n), "launches": top_n,
        "share_of_step": round(top_ms / prof_ms, 4),
        "step": {"achieved": round((total_out + total_comp) / (ms_per_step / 1e3) / 1e9, 1),
                 "frac": round((total_out + total_comp) / (ms_per_step / 1e3) / 1e9 / peak, 4),
                 "algorithmic_bytes": total_out + total_comp},
        "kinds": {k: {"ms": round(v[0], 4), "launches": v[2], "gbs": round(v[1] / (v[0] / 1e3) / 1e9, 1)}
                  for k, v in sorted(by_kind.items(), key=lambda kv: -kv[1][0])},
    }

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

    # ---- CPU baseline (rank 0, N=1 only): the same frames on the host cores
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        dec = CpuDecoder()
        idx = cpu_sample(spec, osizes, total_out // 4, args.seed)
        out_c = np.zeros(obytes, np.uint8)
        cpu_decode_pass(dec, frames_np, foffs, fsizes, out_c, ooffs, osizes, idx[:16], threads)
        reps, secs, nb = 0, 0.0, 0
        while reps < 3 or secs < 3.0:
            t, b = cpu_decode_pass(dec, frames_np, foffs, fsizes, out_c, ooffs, osizes, idx, threads)
            secs += t
            nb += b
            reps += 1
            if reps >= 20:
                break
        for i in idx:
            if not np.array_equal(out_c[ooffs[i]:ooffs[i] + osizes[i]], host_in[ooffs[i]:ooffs[i] + osizes[i]]):
                raise RuntimeError("CPU decode mismatch on frame %d" % i)
        cpu = {"value": round(nb / secs / 1e9, 4), "unit": "GB/s", "cores": threads, "kind": dec.kind,
               "sample": "%d of %d frames (%.1f MiB decoded), %d passes, %d threads" % (
                   len(idx), n_frames, sum(osizes[i] for i in idx) / 2**20, reps, threads)}

    srt = sorted(step_ms)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded random walks)",
        "config": {"workload": WORKLOAD, "frames": n_frames, "decoded_bytes": total_out,
                   "compressed_bytes": total_comp, "ratio": round(total_out / total_comp, 3),
                   "graphs": "delta->tsplit->FSE | delta->bitpack->Huffman", "format_version": 23,
                   "checksums": "content+compressed, verified on device", "l2": "inputs larger than L2 (no flush)"},
        "frac_hbm": round(value / ws / peak, 4),
        "p50_ms": round(statistics.median(step_ms), 4),
        "p99_ms": round(srt[min(len(srt) - 1, int(round(0.99 * (len(srt) - 1))))], 4),
        "plain": plain,
        "encode": {"value": round(enc_gbs, 3), "unit": "GB/s", "note": "batched compress, host decisions included"},
        "roofline": roofline,
        "cpu_baseline": cpu,
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
