"""Double-word (float-float) arithmetic used by the GPU solves.

The header mlcp_gb300/csrc/dword.cuh is compiled for the host with
-ffp-contract=off and checked against long double on 200k seeded operands.
Bounds (relative error, as -log2): the published bounds for the algorithms
(Joldes, Muller, Popescu, ACM TOMS 2017: DWPlusDW <= 3u^2, DWTimesDW <= 5u^2
with u = 2^-24) give about 46 bits (the sloppy sum, Alg. 5, is measured against
|a| + |b|, the form of its bound); the Newton-step reciprocal and square
root lose one or two more.  The device reciprocal seed (rcp.approx, 2^-23)
is one bit coarser than the host's rounded division, so the device ends
about a bit lower on rcp/div; the GPU ALS tests cover that path.  The
compensated dot product and sum (acc_*, Ogita-Rump-Oishi Dot2 with
double-word operands) are measured on 1-40 terms against sum |x_i y_i|; their
bound grows like n u^2, so 40 terms stay above 42 bits.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

BITS = {"add": 45.0, "add_sloppy": 45.0, "mul": 45.0, "fma": 44.5, "rcp": 45.0, "div": 44.0, "sqrt": 44.0,
        "add_f": 45.0, "mul_f": 45.0, "from_double": 47.0, "acc_dot": 42.0, "acc_sum": 42.0}


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("dword") / "dword_check")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-I", os.path.join(ROOT, "mlcp_gb300", "csrc"),
                    os.path.join(HERE, "dword_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {line.split()[0]: float(line.split()[1]) for line in out.strip().splitlines()}


@pytest.mark.parametrize("op", sorted(BITS))
def test_dword_accuracy(results, op):
    assert results[op] >= BITS[op], (op, results[op])
