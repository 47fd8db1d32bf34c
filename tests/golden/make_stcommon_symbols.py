"""Writes reference_stcommon_symbols.txt: the C names that the reference's
Python bindings (python/sixtracklib/stcommon.py) bind from its shared
library outside the CUDA / OpenCL sections, one per line.  Run where the
reference sources are present:

    python tests/golden/make_stcommon_symbols.py /root/reference
"""

import os
import re
import sys

root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
src = open(os.path.join(root, "python", "sixtracklib", "stcommon.py")).read()
core = src.split("if SIXTRACKLIB_MODULES.get(", 1)[0]
names = sorted(set(re.findall(r"sixtracklib\.(st_\w+)", core)))
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_stcommon_symbols.txt")
with open(out, "w") as f:
    f.write("\n".join(names) + "\n")
print(f"{len(names)} names -> {out}")
