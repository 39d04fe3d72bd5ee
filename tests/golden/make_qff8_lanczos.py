"""Known answer for the three-layer tree test: the 10 lowest eigenvalues of
the synthetic quartic force field hoplist.synthetic_qff(8, 4, seed=11) (8
modes of 4 harmonic-oscillator functions, 4^8 = 65536 product states) by
ARPACK Lanczos (scipy eigsh) with H applied term by term on the full
direct-product grid.

    python tests/golden/make_qff8_lanczos.py      # about 40 s

writes tests/golden/qff8_n4_seed11_lowest10.json."""
import json
import os
import sys

import numpy as np
import scipy.sparse.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from mlcp_gb300 import hoplist as H  # noqa: E402

D, N1, SEED, K = 8, 4, 11, 10


def main():
    hl = H.synthetic_qff(D, N1, seed=SEED, eigenbasis=False)
    cache = H.operator_cache(hl)
    shape = (N1,) * D
    N = N1 ** D
    op = sla.LinearOperator((N, N), matvec=lambda x: H.apply_direct(hl, x.reshape(shape), cache).ravel(),
                            dtype=np.float64)
    w = np.sort(sla.eigsh(op, k=K, which="SA", tol=1e-12)[0])
    out = {"system": f"hoplist.synthetic_qff({D}, {N1}, seed={SEED}) in the primitive HO basis",
           "method": "ARPACK Lanczos (scipy.sparse.linalg.eigsh, which=SA, tol=1e-12), full 4^8 basis",
           "eigenvalues": [float(x) for x in w]}
    with open(os.path.join(HERE, "qff8_n4_seed11_lowest10.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(out["eigenvalues"])


if __name__ == "__main__":
    main()
