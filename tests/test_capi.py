"""The C-ABI library builds, loads without a GPU and exports every entry
point that include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        for m in re.finditer(r"MLCP_API\s+[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_reference_entry_points():
    names = declared_symbols()
    for ref in ("intertwinecpp_", "alscpp_", "intwdevicemem_"):
        assert ref in names


def test_library_exports_declared_symbols():
    from mlcp_gb300 import _lib
    path = _lib.load().__dict__.get("_name") or _lib.lib_path()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert declared_symbols() <= exported


def test_library_links_no_oracle():
    """The product library does not depend on the oracle."""
    from mlcp_gb300 import _lib
    out = subprocess.run(["nm", "-D", _lib.lib_path()], capture_output=True, text=True).stdout
    assert "orc_" not in out
    deps = subprocess.run(["ldd", _lib.lib_path()], capture_output=True, text=True).stdout
    assert "oracle" not in deps
