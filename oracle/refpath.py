"""Where the reference's source tree lies, for the recipes and tests that
compile or read it: $OZL_REFERENCE, else the REF default of oracle/ref.mk.
Test infrastructure only; the GPU library never reads the reference."""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root():
    env = os.environ.get("OZL_REFERENCE")
    if env:
        return env
    with open(os.path.join(HERE, "ref.mk")) as f:
        m = re.search(r"^REF\s*\?=.*?(/[^\s,)]+)", f.read(), flags=re.M)
    return m.group(1) if m else ""


def reference_present():
    root = reference_root()
    return bool(root) and os.path.isdir(os.path.join(root, "src", "openzl"))
