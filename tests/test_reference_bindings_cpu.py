"""Which of the C names the reference's Python bindings bind
(tests/golden/reference_stcommon_symbols.txt, from
python/sixtracklib/stcommon.py outside its CUDA / OpenCL sections) this
library exports.  The reference's generic device-controller layer
(NS(Controller), NS(Argument), NS(NodeInfo), NS(NodeId), NS(KernelConfig))
is not part of this path; every other name is exported, except those listed
in tests/golden/stcommon_symbols_not_bound.txt.  A name that becomes
exported must leave that list, so the list only shrinks."""

import ctypes as C
import os

from sixtracklib_gb300 import _native

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
OUT_OF_SCOPE = ("st_Controller_", "st_Argument_", "st_NodeInfo_", "st_NodeId_",
                "st_KernelConfig_")


def _names(fname):
    with open(os.path.join(GOLDEN, fname)) as f:
        return {l.strip() for l in f if l.strip() and not l.startswith("#")}


def test_reference_binding_names_are_exported():
    _native.load()
    lib = C.CDLL(_native.lib_path())
    wanted = {n for n in _names("reference_stcommon_symbols.txt")
              if not n.startswith(OUT_OF_SCOPE)}
    not_bound = _names("stcommon_symbols_not_bound.txt")
    exported = {n for n in wanted if hasattr(lib, n)}
    assert not_bound <= wanted
    assert wanted - exported == not_bound, (
        f"newly missing: {sorted(wanted - exported - not_bound)}; "
        f"now exported (drop from the list): {sorted(not_bound & exported)}")
    assert len(exported) >= 245
