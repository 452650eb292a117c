"""Serving loop's shared HBM pool (host logic, no GPU): the first-fit
allocator that admits requests by free pool bytes, checked against a byte-map
model on random take/give sequences (tests/native/pool_blocks_check.cpp)."""
import os
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("pool") / "pool_blocks_check")
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-I",
           os.path.join(ROOT, "openzl_gb300", "csrc"), os.path.join(ROOT, "tests", "native", "pool_blocks_check.cpp"),
           "-o", exe]
    subprocess.check_call(cmd)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_first_fit_pool_against_model(checker, seed):
    r = subprocess.run([checker, str(seed)], capture_output=True, text=True)
    assert r.returncode == 0 and "bad=0" in r.stdout, (r.stdout[-2000:], r.stderr[-2000:])
    takes = int(r.stdout.split("takes=")[1].split()[0])
    fails = int(r.stdout.split("fails=")[1].split()[0])
    assert takes > 1000 and fails > 10, r.stdout  # both outcomes exercised
