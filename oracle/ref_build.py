"""Recipe for the reference's own FP64 CUDA library (test infrastructure).

The reference implements the power-iteration hot path as CUDA C++
(src/intertwining.cu, src/als.cu, src/intertw_mvp.cu, src/intertw_lcv.cu,
src/modvecvec.cu, src/cpvector.cu, src/hoplist.cu, src/matrix.cu,
src/linalg.cu, src/utils.cu).  Its shipped build is double precision
(Makefile:17 ``USEDOUBLES = yes`` -> ``-DUSE_DOUBLES=1``): this is the plain
FP64 GPU form that parity and speed are measured against.  This recipe builds
that library, unchanged apart from one fix, so that the tests and the
benchmark can run it beside ``libmlcp_gb300``.

Two steps, because the machine that holds the reference tree has no GPU and
the machine with the GPU holds no reference tree (and runs another CPU
architecture, so nothing compiled here runs there):

``stage()``  (where ``/root/reference`` exists) copies the ten ``.cu`` files
and their headers into ``oracle/_ref/src`` (git-ignored: reference sources
never enter this repository's history) and applies the one fix below.

``build()``  (where ``oracle/_ref/src`` and nvcc exist) compiles them as the
reference's Makefile does (``-dc``, ``-default-stream per-thread``,
``-Xcompiler -fopenmp``, ``-O3``, ``-DUSE_DOUBLES=1``; Makefile:117-156,
302-303), for sm_103a, into ``oracle/_ref/libmlcpref.so`` linked against
cuSOLVER/cuBLAS (Makefile:144).

The fix: ``intwvars::init`` (src/als.cu:29-56) allocates ``nbas`` with the
rank as its length and copies that many entries from the vector's ``nbas``,
but ``ITERATE_ALS`` and ``POW_ALS`` index it by mode (src/als.cu:1052,
src/intertw_mvp.cu:473).  With more modes than the rank (the 30-mode ALS
benchmark at rank 20) the later entries are uninitialised and the mode loops
run over garbage sizes; with fewer, the copy reads past the caller's array.
The staged copy sizes and fills it by the number of modes.  Nothing else is
changed; ``stage()`` refuses to run if the text it patches is not found
exactly once.

The reference calls ``cudaDeviceReset()`` at the end of every entry point
(src/intertwining.cu:175,200), which would destroy any other CUDA state in
the calling process, so the library is only ever loaded by the runner
``oracle/ref_run.py`` in a child process.
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_TREE = "/root/reference"
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libmlcpref.so")
MANIFEST = os.path.join(SRC, "MANIFEST.json")

CU_FILES = ["utils.cu", "matrix.cu", "linalg.cu", "cpvector.cu", "hoplist.cu", "modvecvec.cu", "als.cu",
            "intertw_mvp.cu", "intertw_lcv.cu", "intertwining.cu"]

# (file, exact text, replacement): the nbas sizing fix of intwvars::init
PATCHES = [
    ("als.cu", "   nbas = new int [rrk];\n", "   nbas = new int [ndof];\n"),
    ("als.cu", "   for (int i=0;i<rrk;i++){\n       nbas[i]=Q_h.nbas[i];\n",
     "   for (int i=0;i<ndof;i++){\n       nbas[i]=Q_h.nbas[i];\n"),
]

FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-DUSE_DOUBLES=1", "-default-stream", "per-thread",
         "-Xcompiler", "-fopenmp", "-Xcompiler", "-fPIC", "-Wno-deprecated-gpu-targets"]


def _sha(path: str) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def staged() -> bool:
    return os.path.exists(MANIFEST)


def stage(tree: str = REF_TREE) -> bool:
    """Copy the reference's CUDA sources into oracle/_ref/src and apply the
    nbas fix.  Returns False (and does nothing) when the tree is absent."""
    src_dir = os.path.join(tree, "src")
    if not os.path.isdir(src_dir):
        return False
    names = CU_FILES + sorted(os.path.basename(p) for p in glob.glob(os.path.join(src_dir, "*.h")))
    want = {n: _sha(os.path.join(src_dir, n)) for n in names}
    if staged():
        with open(MANIFEST) as f:
            if json.load(f).get("sources") == want:
                return True
    os.makedirs(SRC, exist_ok=True)
    for n in names:
        shutil.copyfile(os.path.join(src_dir, n), os.path.join(SRC, n))
    for fname, old, new in PATCHES:
        p = os.path.join(SRC, fname)
        with open(p) as f:
            text = f.read()
        if text.count(old) != 1:
            raise RuntimeError(f"reference patch target not found exactly once in {fname}: {old!r}")
        with open(p, "w") as f:
            f.write(text.replace(old, new))
    with open(MANIFEST, "w") as f:
        json.dump({"tree": tree, "sources": want, "patches": [[p[0], p[1], p[2]] for p in PATCHES],
                   "flags": FLAGS}, f, indent=1)
    return True


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False) -> str | None:
    """Compile the staged sources into oracle/_ref/libmlcpref.so.  Returns the
    library path, or None when no sources are staged."""
    if not staged():
        return None
    srcs = [os.path.join(SRC, n) for n in CU_FILES]
    hdrs = glob.glob(os.path.join(SRC, "*.h"))
    if not force and not _stale(LIB, srcs + hdrs + [MANIFEST, __file__]):
        return LIB
    cc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = [cc, *FLAGS, "-I", SRC, "-dc", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for reference {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    # shared CUDA runtime, found through an rpath to the toolkit's libraries,
    # so that the runner can create the context before timing a call
    libdir = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), "lib64")
    cmd = [cc, *FLAGS, "-shared", "-rdc=true", "-cudart", "shared", "-o", tmp, *objs, "-lcusolver", "-lcublas",
           "-lgomp", "-Xlinker", "-rpath", "-Xlinker", libdir]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link of the reference library failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print("staged:", stage())
    if "--build" in sys.argv:
        print(build(force="--force" in sys.argv))
