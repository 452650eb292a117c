"""Frame-header summaries: the host parse (ozl_frame_info) against the frame
calls it summarizes, and the device parse (ozl_gpu_frame_info) against the
host's records, byte for byte, on the reference's frames (format versions
8-23, several outputs) and on truncated and corrupted copies."""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, read_frame


def _all_cases():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.zl")))


def _variants(frame, rng):
    """The frame, every truncation inside its first 48 bytes, its header end
    (+-1), and copies with random bytes of the header flipped."""
    fr = bytes(frame)
    out = [fr]
    for n in range(0, min(len(fr), 48)):
        out.append(fr[:n])
    for k in range(12):
        b = bytearray(fr)
        i = int(rng.integers(0, min(len(b), 24)))
        b[i] ^= int(rng.integers(1, 256))
        out.append(bytes(b))
    return out


def _record_bytes(info):
    return ctypes.string_at(ctypes.addressof(info), ctypes.sizeof(info))


def test_host_frame_info_matches_frame_calls():
    """Host summary of every reference frame: parse succeeds, output 0 and the
    destination extent agree with the frame-information calls."""
    import openzl_gb300 as oz

    assert ctypes.sizeof(oz.FrameHeaderInfo) == 48
    for case in _all_cases():
        fr = read_frame(case)
        info = oz.frame_header_info(fr)
        lay, ext = oz.frame_outputs(fr)
        assert info.status == 0, case
        assert info.nbOutputs == len(lay), case
        assert info.extent == ext, case
        assert info.output0Bytes == lay[0]["size"], case
        assert 8 <= info.formatVersion <= 23, case
        assert info.headerBytes < len(fr), case
    # errors: empty, too small, bad magic
    assert oz.frame_header_info(b"").status == 3
    assert oz.frame_header_info(b"\x00" * 4).status == 3
    bad = bytearray(read_frame(_all_cases()[0]))
    bad[3] ^= 0x40
    assert oz.frame_header_info(bytes(bad)).status == 60


@pytest.mark.gpu
def test_device_frame_info_equals_host(gpu_lib):
    """Every record the device writes equals the host's for the same bytes."""
    import torch
    import openzl_gb300 as oz

    rng = np.random.default_rng(77)
    frames = []
    for case in _all_cases():
        frames.extend(_variants(read_frame(case), rng))
    n = len(frames)
    # device copies (each at least 16 bytes, so an empty frame has an address)
    dev = [torch.from_numpy(np.frombuffer(f + bytes(16), np.uint8).copy()).to("cuda") for f in frames]
    ptrs = torch.tensor([d.data_ptr() for d in dev], dtype=torch.int64, device="cuda")
    sizes = torch.tensor([len(f) for f in frames], dtype=torch.int64, device="cuda")
    out = torch.zeros(n * 48, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    assert oz.frame_header_info_device(ptrs.data_ptr(), sizes.data_ptr(), n, out.data_ptr(), s.cuda_stream) == n
    s.synchronize()
    got = out.cpu().numpy().tobytes()
    statuses = set()
    for i, f in enumerate(frames):
        want = _record_bytes(oz.frame_header_info(f))
        assert got[48 * i:48 * i + 48] == want, (i, len(f))
        statuses.add(oz.frame_header_info(f).status)
    # the variants reach the parse's error paths, not just its success
    assert {0, 3, 60} <= statuses, statuses
