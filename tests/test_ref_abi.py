"""A C caller built against the reference's own public headers links and runs
against libopenzl_gb300.so, and prints the same results as the same program
linked against the reference library (compiled here by oracle/ref.mk).

Skipped where the reference's headers are absent. CPU only: the caller uses
entry points that need no GPU (frame inspection, ZL_Report through the
headers' inline accessors, parameters, host-side refusals, graph building,
custom-codec registration)."""
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT
from oracle.refpath import reference_present, reference_root

pytestmark = pytest.mark.skipif(not reference_present(), reason="reference sources not present")

SRC = os.path.join(ROOT, "tests", "native", "ref_header_caller.c")
FRAME = os.path.join(GOLDEN, "walk_u32_1mib_dz_tsplit_fse.zl")
REF_LIB_DIR = os.path.join(ROOT, "oracle", "_ref")
# malformed-frame paths: the reference reports most of them as GENERIC with a
# "corruption" message, this library as ZL_ErrorCode_corruption; only the
# error flag is compared on these lines
CODE_MAY_DIFFER = ("getCompressedSize(truncated)",)


def _build_and_run(tmp_path, name, libdir, lib, extra=()):
    exe = os.path.join(str(tmp_path), name)
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(reference_root(), "include"), SRC,
           "-L", libdir, "-l" + lib, "-Wl,-rpath," + libdir, "-o", exe] + list(extra)
    subprocess.check_call(cmd)
    out = subprocess.run([exe, FRAME], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout.splitlines()


def _split(lines):
    k = lines.index("-- custom codecs")
    shared = {}
    for l in lines[:k]:
        key, val = l.split(": ", 1)
        if key in CODE_MAY_DIFFER:
            val = val.split(" code=")[0]
        shared[key] = val
    custom = dict(l.split(": ", 1) for l in lines[k + 1:])
    return shared, custom


@pytest.fixture(scope="module")
def ours(tmp_path_factory):
    from openzl_gb300 import build, library_path

    build.build()
    return _split(_build_and_run(tmp_path_factory.mktemp("ours"), "caller_ours",
                                 os.path.dirname(library_path()), "openzl_gb300"))


def test_caller_against_this_library(ours):
    shared, custom = ours
    assert shared["getDecompressedSize"] == "err=0 code=0 value=1048576"
    assert shared["getCompressedSize"] == "err=0 code=0 value=%d" % os.path.getsize(FRAME)
    assert shared["FrameInfo_getFormatVersion"] == "err=0 code=0 value=23"
    assert shared["DCtx_getParameter(sticky)"] == "1"
    assert shared["DCtx_getParameter(sticky) after reset"] == "0"
    assert shared["DCtx_decompress(8-byte dst)"] == "err=1 code=5 value=0"
    assert shared["CCtx_compressTypedRef(no formatVersion)"] == "err=1 code=61 value=0"
    # custom codecs are refused, and the opaque pointers are released once each
    assert custom["DCtx_registerTypedDecoder"] == "err=1 code=81 value=0"
    assert custom["Compressor_registerTypedEncoder illegal"] == "1"
    assert custom["opaque released before free"] == "2"
    assert custom["opaque released after free"] == "2"


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_LIB_DIR, "libozl_ref.so")),
                    reason="reference library not built here")
def test_caller_prints_the_same_results_against_the_reference(ours, tmp_path):
    ref_shared, ref_custom = _split(_build_and_run(tmp_path, "caller_ref", REF_LIB_DIR, "ozl_ref", ["-lm"]))
    shared, _ = ours
    assert shared == ref_shared
    # the reference registers the codecs and releases the pointers when the
    # contexts are freed
    assert ref_custom["opaque released after free"] == "2"
