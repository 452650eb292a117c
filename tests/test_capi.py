"""The C-ABI library: builds for sm_103a, exports every declared entry point,
and its host-only entry points (frame inspection, planning) work without a
GPU."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, read_frame


@pytest.fixture(scope="module")
def lib():
    from openzl_gb300 import build

    build.build()
    import openzl_gb300

    return openzl_gb300.library()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(inc, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b((?:ZL|ozl)_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    from openzl_gb300 import library_path

    out = subprocess.run(["nm", "-D", "--defined-only", library_path()], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    decl = declared_symbols()
    assert len(decl) >= 20
    missing = decl - exported
    assert not missing, missing


def test_frame_inspection_on_golden_frames(lib, manifest):
    import openzl_gb300 as oz

    for m in manifest:
        fr = read_frame(m["case"])
        width = m["elt_width"] or 1
        assert oz.get_decompressed_size(fr) == m["n"] * width, m["case"]
        # planning walks every block header; the frame ends at its marker byte
        assert oz.get_compressed_size(fr) == len(fr), m["case"]


def test_inspection_errors_without_gpu(lib):
    import openzl_gb300 as oz

    with pytest.raises(oz.ZLError):
        oz.get_decompressed_size(b"\x00" * 16)
    bad = bytearray(read_frame("walk_u32_1mib_dz_tsplit_fse"))
    bad[3] ^= 0x10
    with pytest.raises(oz.ZLError) as e:
        oz.get_compressed_size(bytes(bad))
    assert e.value.code == 60
    trunc = read_frame("walk_u32_1mib_dz_tsplit_fse")[:100]
    with pytest.raises(oz.ZLError):
        oz.get_compressed_size(trunc)
