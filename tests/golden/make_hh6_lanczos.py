"""Known answer for the power-cycle workload: the 40 lowest eigenvalues of the
modified Henon-Heiles Hamiltonian of the benchmark (D = 6 modes, lambda =
0.111803, 10 harmonic-oscillator functions per mode) on the full 10^6
direct-product basis, by ARPACK Lanczos (scipy eigsh) with H applied term by
term as Kronecker products of the operator list's per-mode matrices.

    python tests/golden/make_hh6_lanczos.py      # about 6 minutes on 8 cores

writes tests/golden/hh6_n10_lowest40.json."""
import json
import os
import sys

import numpy as np
import scipy.sparse.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from mlcp_gb300 import hoplist as H  # noqa: E402


def main():
    hl = H.henon_heiles(D=6, n=10, lam=0.111803)
    nb = [int(x) for x in hl.nbas]
    N = int(np.prod(nb))
    terms = []
    for t in range(hl.nterms):
        ops = [(d, hl.operator(t, d)) for d in range(hl.ndof) if not np.allclose(hl.operator(t, d), np.eye(nb[d]))]
        terms.append((float(hl.coef[t]), ops))

    def matvec(x):
        x = np.asarray(x).reshape(nb)
        y = np.zeros_like(x)
        for a, ops in terms:
            z = x
            for d, O in ops:
                z = np.moveaxis(np.tensordot(O, z, axes=([1], [d])), 0, d)
            y += a * z
        return y.ravel()

    op = sla.LinearOperator((N, N), matvec=matvec, dtype=np.float64)
    vals = np.sort(sla.eigsh(op, k=40, which="SA", tol=1e-12, ncv=120, return_eigenvectors=False))
    out = {"workload": "modified Henon-Heiles, D=6, lambda=0.111803, 10 HO functions per mode (10^6 basis)",
           "method": "ARPACK Lanczos (scipy.sparse.linalg.eigsh, tol 1e-12, ncv 120)",
           "eigenvalues": [float(v) for v in vals]}
    with open(os.path.join(HERE, "hh6_n10_lowest40.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(vals)


if __name__ == "__main__":
    main()
