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


def test_sortvecscpp_matches_oracle():
    """sortvecscpp_ is host code: checked here without a GPU."""
    import numpy as np
    import oracle
    from mlcp_gb300 import intertwine as IT
    rng = np.random.default_rng(5)
    nbas = [3, 4, 2]
    rk, nbloc, nD = 3, 9, 9
    for trial in range(6):
        Q, qc = rng.normal(size=(rk * nbloc, nD)), rng.uniform(0.2, 1.0, rk * nbloc)
        eig = rng.normal(size=nbloc) * 3
        if trial == 5:
            eig = np.sort(np.abs(eig))  # already in order: nothing moves
        nconv = int(rng.integers(0, nbloc + 1))
        eref = float(rng.normal()) if trial < 5 else 0.0
        gb, gc, ge, gn = IT.sort_vecs(Q, qc, nbas, rk, eig, nconv, eref)
        ob, oc, oe, on = oracle.sort_vecs(Q, qc, rk, eig, nconv, eref)
        assert np.array_equal(gb, ob) and np.array_equal(gc, oc) and np.array_equal(ge, oe) and gn == on
