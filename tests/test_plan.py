"""Decode planner (host logic, no GPU): every golden frame plans and lays out
with every task's pointers and lengths inside the allocations they address."""
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("plan") / "plan_check")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-I",
           os.path.join(ROOT, "openzl_gb300", "csrc"), os.path.join(ROOT, "tests", "native", "plan_check.cpp"),
           os.path.join(ROOT, "openzl_gb300", "csrc", "dec_plan.cpp"), "-o", exe]
    subprocess.check_call(cmd)
    return exe


def test_every_golden_layout_is_in_bounds(checker, manifest):
    for m in manifest:
        r = subprocess.run([checker, os.path.join(GOLDEN, m["case"] + ".zl")], capture_output=True, text=True)
        assert r.returncode == 0 and "bad=0" in r.stdout, (m["case"], r.stdout[-2000:], r.stderr[-2000:])


def test_fused_pipeline_shape(checker):
    """delta <- zigzag <- view <- transpose fuse into one planes-sourced pass
    that runs after the entropy level, and checksums run last."""
    r = subprocess.run([checker, os.path.join(GOLDEN, "walk_u32_1mib_dz_tsplit_fse.zl")], capture_output=True,
                       text=True)
    out = r.stdout
    assert "np n=262144 w=4 mode=1 zz=1 delta=1" in out
    kinds = [l.split()[1] for l in out.splitlines() if l.strip().startswith("launch")]
    assert kinds == ["kind=1", "kind=2", "kind=8", "kind=9"], kinds


def test_mutated_frames_are_refused_or_in_bounds(checker, manifest, manifest_multi):
    """Malformed input: 300 mutated copies of every golden frame (bytes
    flipped, set to 0x00 or 0xFF, truncated; half the mutations in the
    headers) are each refused by the planner or planned with every task's
    pointers and lengths inside their allocations, under ASan/UBSan."""
    planned = refused = 0
    for k, m in enumerate(list(manifest) + list(manifest_multi)):
        r = subprocess.run([checker, os.path.join(GOLDEN, m["case"] + ".zl"), "--fuzz", "300", str(k + 1)],
                           capture_output=True, text=True)
        assert r.returncode == 0 and "bad=0" in r.stdout, (m["case"], r.stdout[-2000:], r.stderr[-2000:])
        planned += int(r.stdout.split("planned=")[1].split()[0])
        refused += int(r.stdout.split("refused=")[1].split()[0])
    assert planned > 1000 and refused > 1000, (planned, refused)  # both outcomes exercised


def test_multi_output_layouts_in_bounds(checker, manifest_multi):
    """Frames of several outputs: each output and, for the content checksum,
    each gathered block lie inside their allocations."""
    for m in manifest_multi:
        r = subprocess.run([checker, os.path.join(GOLDEN, m["case"] + ".zl")], capture_output=True, text=True)
        assert r.returncode == 0 and "bad=0" in r.stdout, (m["case"], r.stdout[-2000:], r.stderr[-2000:])


def test_parallel_build_equals_serial(tmp_path, manifest, manifest_multi):
    """The planner's parallel build (runs of frames on 4 threads, joined)
    gives the serial plan and the same task descriptors, byte for byte, on
    every golden frame (single and multi-output) repeated to 600 frames."""
    exe = str(tmp_path / "plan_parallel_check")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-pthread", "-fsanitize=address,undefined", "-I",
           os.path.join(ROOT, "openzl_gb300", "csrc"), os.path.join(ROOT, "tests", "native", "plan_parallel_check.cpp"),
           os.path.join(ROOT, "openzl_gb300", "csrc", "dec_plan.cpp"), "-o", exe]
    subprocess.check_call(cmd)
    files = [os.path.join(GOLDEN, m["case"] + ".zl") for m in manifest + manifest_multi]
    r = subprocess.run([exe] + files, capture_output=True, text=True)
    assert r.returncode == 0 and "bad=0" in r.stdout, (r.stdout[-2000:], r.stderr[-2000:])
