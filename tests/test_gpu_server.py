"""Serving loop: requests of mixed kinds and sizes give the same bytes when
run alone (one request in the system at a time) and in the mix (all queued
at once over several workers), and both equal the expected result (decoded
input; the reference's frame through the oracle). Errors stay with their own
request."""
import time

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _requests(seed=7):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(48):
        w = int(rng.choice([1, 2, 4, 8]))
        n = int(np.exp(rng.uniform(np.log(300), np.log(400000)))) // w + 1
        dt = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[w]
        a = (1000 + np.cumsum(rng.integers(-int(rng.integers(1, 5000)), 5000, n))).astype(dt)
        recipe = 3 if k % 3 else 4
        if k % 5 == 0:
            reqs.append(("c", a, w, recipe, oracle.compress(recipe, a, w)))
        else:
            reqs.append(("d", oracle.compress(recipe, a, w), w, recipe, a))
    return reqs


def _submit(srv, r):
    kind, x, w, recipe, want = r
    if kind == "d":
        out = np.zeros(max(want.nbytes, 1), np.uint8)
        return srv.submit_decompress(x, out), out
    out = np.zeros(2 * x.nbytes + 1024, np.uint8)
    return srv.submit_compress(x, w, recipe, out), out


def _collect(srv, n, timeout=120):
    got = {}
    t0 = time.time()
    while len(got) < n and time.time() - t0 < timeout:
        for i, code, val, lat in srv.poll(wait_ms=100):
            got[i] = (code, val, lat)
    return got


def test_alone_equals_mix_equals_expected(gpu_lib):
    import openzl_gb300 as oz

    reqs = _requests()
    srv = oz.Server(hbm_budget=1 << 30, workers=3)
    alone = []
    for r in reqs:
        i, out = _submit(srv, r)
        res = _collect(srv, 1)
        code, val, lat = res[i]
        assert code == 0, (r[0], code)
        alone.append(out[:val].tobytes())
    ids, outs = [], []
    for r in reqs:
        i, out = _submit(srv, r)
        ids.append(i)
        outs.append(out)
    res = _collect(srv, len(reqs))
    st = srv.stats()
    srv.close()
    assert len(res) == len(reqs)
    # the workers' statistics count every request once
    assert st["decode_requests"] + st["encode_requests"] == 2 * len(reqs), st
    assert st["decode_batches"] >= 1 and st["decode_plan_s"] > 0 and st["decode_run_s"] > 0, st
    for r, i, out, a in zip(reqs, ids, outs, alone):
        code, val, lat = res[i]
        assert code == 0
        mix = out[:val].tobytes()
        assert mix == a  # tolerance 0: bit-exact alone and in the mix
        kind, x, w, recipe, want = r
        assert mix == want.tobytes()
        assert lat > 0


def test_errors_stay_with_their_request(gpu_lib):
    import openzl_gb300 as oz

    reqs = _requests(9)[:12]
    srv = oz.Server(hbm_budget=64 << 20, workers=2)
    ids = []
    outs = []
    for k, r in enumerate(reqs):
        kind, x, w, recipe, want = r
        if kind == "d" and k == 3:
            bad = x.copy()
            bad[len(bad) // 2] ^= 0x5A
            out = np.zeros(want.nbytes, np.uint8)
            ids.append(srv.submit_decompress(bad, out))
        else:
            i, out = _submit(srv, r)
            ids.append(i)
        outs.append(out)
    big = np.zeros(40 << 20, np.uint8)
    big_out = np.zeros(1, np.uint8)
    big_id = srv.submit_compress(big, 0, 0, big_out)  # larger than one 32 MiB arena
    res = _collect(srv, len(ids) + 1)
    srv.close()
    assert res[big_id][0] == 4  # srcSize_tooLarge
    for k, (r, i, out) in enumerate(zip(reqs, ids, outs)):
        code, val, _ = res[i]
        if k == 3 and r[0] == "d":
            assert code != 0
        else:
            assert code == 0
            assert out[:val].tobytes() == r[4].tobytes()


def test_one_request_may_use_the_whole_budget(gpu_lib):
    """Admission draws on one shared budget: a request larger than the
    budget's per-worker share but within the budget runs (after the smaller
    requests ahead of it free their memory), and the requests around it
    still run and stay correct."""
    import openzl_gb300 as oz

    rng = np.random.default_rng(3)
    budget = 96 << 20
    srv = oz.Server(hbm_budget=budget, workers=4)  # per-worker share 24 MiB
    big = (1000 + np.cumsum(rng.integers(-900, 901, 5 << 20))).astype(np.uint32)  # 20 MiB in, 20 MiB out
    big_frame = oracle.compress(3, big, 4)
    small = [_requests(21)[k] for k in range(10)]
    ids, outs, wants = [], [], []
    for r in small[:5]:
        i, out = _submit(srv, r)
        ids.append(i), outs.append(out), wants.append(r[4])
    big_out = np.zeros(big.nbytes, np.uint8)
    big_id = srv.submit_decompress(big_frame, big_out)
    for r in small[5:]:
        i, out = _submit(srv, r)
        ids.append(i), outs.append(out), wants.append(r[4])
    res = _collect(srv, len(ids) + 1)
    srv.close()
    assert res[big_id][0] == 0 and res[big_id][1] == big.nbytes
    assert big_out.tobytes() == big.tobytes()
    for i, out, want in zip(ids, outs, wants):
        code, val, _ = res[i]
        assert code == 0 and out[:val].tobytes() == want.tobytes()
