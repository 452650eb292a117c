"""Allocation-free XXH3 entry point (ozl_gpu_xxh3_64_static): the same hash
as the allocating entry point ozl_gpu_xxh3_64 and the CPU oracle, on calls in
a row that share its fixed device scratch; inputs beyond its maximum size are
rejected. The file name makes pytest collect it last, so that it runs both
alone in a fresh process and after every other test."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

SRC_SIZE_TOO_LARGE = 4  # ZL_ErrorCode_srcSize_tooLarge


@pytest.fixture(scope="module")
def data():
    import torch

    rng = np.random.default_rng(2026)
    host = rng.integers(0, 256, (32 << 20) + 64, dtype=np.uint8)
    dev = torch.from_numpy(host).cuda()
    torch.cuda.synchronize()
    return host, dev


LENGTHS = [0, 1, 3, 4, 8, 9, 16, 17, 128, 129, 240, 241, 1023, 1024, 1025, 4103, 65536 + 17, 1 << 20,
           3 * (1 << 20) + 5, 32 << 20]


@pytest.mark.parametrize("offset", [0, 3])
def test_static_matches_allocating_entry_point_twice(gpu_lib, data, offset):
    import openzl_gb300 as oz

    host, dev = data
    for n in LENGTHS:
        if offset + n > host.size:
            continue
        p = dev.data_ptr() + offset
        want = oz.xxh3_64_device(p, n)
        first = oz.xxh3_64_device_static(p, n)
        second = oz.xxh3_64_device_static(p, n)
        assert first == want and second == want, (n, offset)
        if n <= (1 << 20):
            assert first == oracle.xxh3_64(host[offset:offset + n].tobytes()), (n, offset)


def test_static_consecutive_different_inputs(gpu_lib, data):
    """A long input then a short one, and back: no result carries over."""
    import openzl_gb300 as oz

    _, dev = data
    p = dev.data_ptr()
    for n in [5 << 20, 100, 5 << 20, 3000, 0, 5 << 20]:
        assert oz.xxh3_64_device_static(p + 1, n) == oz.xxh3_64_device(p + 1, n), n


def test_static_on_a_side_stream(gpu_lib, data):
    import torch
    import openzl_gb300 as oz

    _, dev = data
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    n = (7 << 20) + 11
    got = oz.xxh3_64_device_static(dev.data_ptr(), n, s.cuda_stream)
    assert got == oz.xxh3_64_device(dev.data_ptr(), n)


def test_static_rejects_sizes_beyond_the_maximum(gpu_lib, data):
    import openzl_gb300 as oz

    _, dev = data
    assert oz.XXH3_STATIC_MAX_LEN == 32 << 20
    with pytest.raises(oz.ZLError) as e:
        oz.xxh3_64_device_static(dev.data_ptr(), oz.XXH3_STATIC_MAX_LEN + 1)
    assert e.value.code == SRC_SIZE_TOO_LARGE
    # the entry point still works after a rejected call
    assert oz.xxh3_64_device_static(dev.data_ptr(), 4096) == oz.xxh3_64_device(dev.data_ptr(), 4096)
