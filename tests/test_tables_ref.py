"""The encoder's table builders (fse_norm.h and huf_tree.h, shared by host
and device; the 16-bit Huffman builder of enc_tables.cpp) against the
reference's own FSE and Huffman table functions, compiled from its sources
(oracle/ref.mk): FSE table log, normalized counts, normalized-count header,
Huffman table log, code lengths and codes (8- and 16-bit symbols), and the
DataStats estimates the codec decision compares (entropy bit for bit) are
equal on random inputs of many shapes (tests/native/tables_ref_check.cpp).
Skipped where the reference build is absent."""
import os
import subprocess

import pytest

from conftest import ROOT

REF_LIB_DIR = os.path.join(ROOT, "oracle", "_ref")

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF_LIB_DIR, "libozl_ref.so")),
                                reason="the reference oracle (oracle/_ref) is not built here")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("tables") / "tables_ref_check")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "openzl_gb300", "csrc"),
           os.path.join(ROOT, "tests", "native", "tables_ref_check.cpp"),
           os.path.join(ROOT, "openzl_gb300", "csrc", "enc_tables.cpp"), "-L" + REF_LIB_DIR, "-lozl_ref",
           "-Wl,-rpath," + REF_LIB_DIR, "-o", exe]
    subprocess.check_call(cmd)
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_table_builders_equal_reference(checker, seed):
    r = subprocess.run([checker, str(seed), "6000"], capture_output=True, text=True)
    assert r.returncode == 0 and "bad=0" in r.stdout, (r.stdout[-3000:], r.stderr[-2000:])
    fse = int(r.stdout.split("fse=")[1].split()[0])
    huf = int(r.stdout.split("huf=")[1].split()[0])
    huf16 = int(r.stdout.split("huf16=")[1].split()[0])
    stats = int(r.stdout.split("stats=")[1].split()[0])
    assert fse > 10000 and huf > 5000 and huf16 > 500 and stats > 500, r.stdout
