"""GPU encode pinned to the reference's own frame bytes.

The golden frames under tests/golden/ were written by the reference
compressor (tests/golden/make_golden.py). Their inputs are seeded, so the
generator re-creates them here without the reference. Every frame not marked
decode-only is compressed again on the GPU, through the batched encoder and
through ZL_CCtx, and its SHA-256 must equal the manifest's sha256_frame: the
hash of the reference's bytes. No hop through the CPU restatement.
"""
import hashlib
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402


def _inputs(manifest):
    """(manifest entry, input array) for every re-encodable golden frame."""
    arrays = {name: arr for name, _, arr, _, *_ in make_golden.build_cases()}
    out = []
    for m in manifest:
        if m.get("decode_only"):
            continue
        name = m["case"][:-5] if m["case"].endswith("_nock") else m["case"]
        out.append((m, np.ascontiguousarray(arrays[name])))
    return out


def test_generator_recreates_every_golden_input(manifest):
    """The seeded generator still yields the exact inputs the reference
    compressed (input hashes recorded in the manifest)."""
    got = _inputs(manifest)
    assert len(got) == 66
    for m, arr in got:
        assert hashlib.sha256(arr.tobytes()).hexdigest() == m["sha256_in"], m["case"]


@pytest.mark.gpu
def test_gpu_batch_encoder_emits_reference_frames(gpu_lib, manifest):
    import torch
    import openzl_gb300 as oz

    cases = _inputs(manifest)
    enc = oz.GpuEncoder()
    bad = []
    for cs in (1, 0):
        sel = [(m, a) for m, a in cases if m["checksums"] == cs]
        srcs = [torch.from_numpy(a.view(np.uint8).copy()).cuda() if a.size else
                torch.zeros(1, dtype=torch.uint8, device="cuda") for _, a in sel]
        caps = [enc.bound(a.nbytes) for _, a in sel]
        dsts = [torch.zeros(c, dtype=torch.uint8, device="cuda") for c in caps]
        sizes = enc.compress_batch([s.data_ptr() for s in srcs],
                                   [a.size if m["elt_width"] else a.nbytes for m, a in sel],
                                   [m["elt_width"] for m, _ in sel], [m["recipe"] for m, _ in sel],
                                   [d.data_ptr() for d in dsts], caps, checksums=bool(cs))
        for (m, _), d, sz in zip(sel, dsts, sizes):
            h = hashlib.sha256(d[:sz].cpu().numpy().tobytes()).hexdigest()
            if h != m["sha256_frame"]:
                bad.append((m["case"], sz, m["frame_bytes"]))
    assert not bad, bad


@pytest.mark.gpu
def test_cctx_emits_reference_frames(gpu_lib, manifest):
    """The same inputs through the reference's own API: a ZL_Compressor graph
    built with the reference's calls, ZL_CCtx_compress / compressTypedRef."""
    import openzl_gb300 as oz
    from test_gpu_compress_api import _graph

    a = oz.api
    bad = []
    for m, arr in _inputs(manifest):
        comp = oz.Compressor()
        comp.select(_graph(oz, comp, m["recipe"]))
        cctx = oz.CCtx()
        cctx.ref_compressor(comp)
        cctx.set_parameter(a.CPARAM_FORMAT_VERSION, 23)
        if not m["checksums"]:
            cctx.set_parameter(a.CPARAM_CONTENT_CHECKSUM, 2)
            cctx.set_parameter(a.CPARAM_COMPRESSED_CHECKSUM, 2)
        got = cctx.compress(arr.tobytes()) if m["elt_width"] == 0 else cctx.compress_numeric(arr)
        if hashlib.sha256(got.tobytes()).hexdigest() != m["sha256_frame"]:
            bad.append((m["case"], got.size, m["frame_bytes"]))
    assert not bad, bad


@pytest.mark.gpu
def test_gpu_encoder_one_frame_per_call_emits_reference_frames(gpu_lib, manifest):
    """Each golden input alone in its own encoder call (no batch neighbours)."""
    import torch
    import openzl_gb300 as oz

    enc = oz.GpuEncoder()
    bad = []
    for m, a in _inputs(manifest):
        src = torch.from_numpy(a.view(np.uint8).copy()).cuda() if a.size else \
            torch.zeros(1, dtype=torch.uint8, device="cuda")
        cap = enc.bound(a.nbytes)
        dst = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        (sz,) = enc.compress_batch([src.data_ptr()], [a.size if m["elt_width"] else a.nbytes], [m["elt_width"]],
                                   [m["recipe"]], [dst.data_ptr()], [cap], checksums=bool(m["checksums"]))
        if hashlib.sha256(dst[:sz].cpu().numpy().tobytes()).hexdigest() != m["sha256_frame"]:
            bad.append(m["case"])
    assert not bad, bad
