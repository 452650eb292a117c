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


def test_frame_info_on_golden_frames(lib, manifest):
    """ZL_FrameInfo (header only, no GPU): version, outputs, type, size."""
    import openzl_gb300 as oz

    types = {"serial": 1, "struct": 2, "numeric": 4}
    for m in manifest:
        fr = read_frame(m["case"])
        fi = oz.FrameInfo(fr)
        v = m.get("format_version", 23)
        assert fi.format_version() == v
        assert fi.num_outputs() == 1
        width = m["elt_width"] or 1
        assert fi.decompressed_size() == m["n"] * width, m["case"]
        assert oz.get_decompressed_size(fr) == m["n"] * width, m["case"]
        assert oz.get_compressed_size(fr) == len(fr), m["case"]
        t = fi.output_type()
        assert t in types.values()
        if v < 21:
            # decode_frameheader.c:448-453: no element counts before v21
            with pytest.raises(oz.ZLError) as e:
                fi.num_elts()
            assert e.value.code == 1
        elif t == 1:
            assert fi.num_elts() == m["n"] * width
        else:
            # decode_frameheader.c:455-467: not known for struct/numeric outputs
            with pytest.raises(oz.ZLError) as e:
                fi.num_elts()
            assert e.value.code == 81


def test_compress_api_errors_before_any_device_work(lib):
    """Parameter and graph errors of ZL_CCtx are reported before any device
    work, with the reference's error codes."""
    import numpy as np
    import openzl_gb300 as oz
    from openzl_gb300 import api

    data = np.arange(1000, dtype=np.uint32)
    comp = oz.Compressor()
    g = comp.node(api.NODE_DELTA_INT, api.GRAPH_STORE)
    comp.select(g)
    cctx = oz.CCtx()
    cctx.ref_compressor(comp)
    with pytest.raises(oz.ZLError) as e:  # formatVersion not set
        cctx.compress_numeric(data)
    assert e.value.code == 61
    cctx.set_parameter(api.CPARAM_FORMAT_VERSION, 22)
    with pytest.raises(oz.ZLError) as e:  # the GPU encoder writes version 23
        cctx.compress_numeric(data)
    assert e.value.code == 60
    cctx.set_parameter(api.CPARAM_FORMAT_VERSION, 23)
    with pytest.raises(oz.ZLError) as e:  # delta takes numeric input
        cctx.compress(data.tobytes())
    assert e.value.code == 54
    # a graph shape the GPU encoder does not implement
    comp2 = oz.Compressor()
    comp2.select(comp2.node(api.NODE_ZIGZAG, api.GRAPH_FSE))
    cctx2 = oz.CCtx()
    cctx2.ref_compressor(comp2)
    cctx2.set_parameter(api.CPARAM_FORMAT_VERSION, 23)
    with pytest.raises(oz.ZLError) as e:
        cctx2.compress_numeric(data)
    assert e.value.code == 30
    # parameters are not sticky by default: formatVersion is gone again
    with pytest.raises(oz.ZLError) as e:
        cctx2.compress_numeric(data)
    assert e.value.code == 61
    # unknown successor graphs are rejected at registration
    assert comp.node(api.NODE_DELTA_INT, 12345) == api.GRAPH_ILLEGAL
    assert lib.ZL_compressBound(1000) == 2 * 1000 + 520


def test_frame_info_and_layout_of_multi_output_frames(lib, manifest_multi):
    """ZL_FrameInfo over frames of several outputs (count, types, sizes; an
    output ID past the last is outputID_invalid), ZL_getDecompressedSize
    refusing them like the reference, and ozl_frame_outputs' layout: outputs
    one after another at 16-byte-aligned offsets, with their element widths."""
    import openzl_gb300 as oz

    for m in manifest_multi:
        fr = read_frame(m["case"])
        fi = oz.FrameInfo(fr)
        outs = m["outputs"]
        assert fi.num_outputs() == len(outs)
        assert fi.format_version() == m.get("format_version", 23)
        for i, o in enumerate(outs):
            assert fi.decompressed_size(i) == o["bytes"], (m["case"], i)
            assert fi.output_type(i) == o["type"], (m["case"], i)
            if o["type"] == 8:  # string counts come with the v21+ header
                assert fi.num_elts(i) == o["n"], (m["case"], i)
        with pytest.raises(oz.ZLError) as e:
            fi.output_type(len(outs))
        assert e.value.code == 22
        if len(outs) > 1:
            # as in the reference, refused only when the output token is 64
            # or more (tests/test_frame_sizes_ref.py pins the values)
            v = m.get("format_version", 23)
            if v > 14 and fr[4 + (1 if v >= 21 else 0)] >= 64:
                with pytest.raises(oz.ZLError) as e:
                    oz.get_decompressed_size(fr)
                assert e.value.code == 23
        assert oz.get_compressed_size(fr) == len(fr)
        lay, extent = oz.frame_outputs(fr)
        end = 0
        for o, l in zip(outs, lay):
            assert l["offset"] % 16 == 0 and l["offset"] >= end
            assert l["size"] == o["bytes"]
            assert l["width"] == (o["elt_width"] or 1) and l["count"] == o["n"]
            end = l["offset"] + l["size"]
            if o["type"] == 8:
                assert l["lens_offset"] % 16 == 0 and l["lens_offset"] >= end
                end = l["lens_offset"] + 4 * o["n"]
        assert extent == end
