"""openzl_gb300: GB300-native OpenZL numeric codec-graph path.

Python host bindings over the C-ABI library (include/openzl_gb300.h). The
GPU path is the only path: importing works anywhere, but every decode call
needs the compiled library (openzl_gb300.build.build()) and a CUDA device,
and raises if either is missing.
"""
from ._lib import (  # noqa: F401
    ZLError,
    DCtx,
    CCtx,
    Compressor,
    FrameInfo,
    GpuBatch,
    GpuEncoder,
    Server,
    decompress,
    xxh3_64_device,
    xxh3_64_device_static,
    XXH3_STATIC_MAX_LEN,
    get_decompressed_size,
    get_compressed_size,
    frame_outputs,
    FrameHeaderInfo,
    frame_header_info,
    frame_header_info_device,
    library,
    library_path,
)
from . import _lib as api  # noqa: F401  (constants: NODE_*, GRAPH_*, CPARAM_*, TYPE_*)
