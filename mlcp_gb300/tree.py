"""A two-layer mode tree solved with the GPU entry points, as the reference's
host walks its layers (src/MLmain.f90 layer loop, UpdateH in
src/Updater.f90:53-106): the benchmark's tree for the modified Henon-Heiles
Hamiltonian -- modes grouped in pairs, each pair solved for its lowest
states, then one top layer over the pair states.

Layer 1 (primitive): every mode in the eigenbasis of its one-mode operator
(src/HamilSetup.f90:570-645).  Layer 2: each pair node's Hamiltonian is its
two one-mode operators plus the coupling inside the pair; the node is solved
by the solver loop (spectral range, GPU power cycles) for `keep` states.
Layer 3: the top node has one mode per pair whose basis is that pair's
states.  Its Hamiltonian is the pairs' eigenvalues as diagonal (eigen)
operators -- what UpdateH stores for the next layer -- plus the couplings
between pairs, whose one-mode factors are carried into the pair bases by
UpdateOperMat (updateopermatcpp_); it is solved for `top_nev` states.
"""
from __future__ import annotations

import numpy as np

from . import hoplist as H
from . import intertwine as IT
from . import solver


def _node_states(hl, nev, rk, ncycle, npow, nals):
    base, coef, eigv, _, hist = solver.solve(hl, nev, rk, ncycle, npow, nals)
    return base, coef, eigv, hist


def hh_tree(D: int = 6, n: int = 10, lam: float = 0.111803, keep: int = 30, top_nev: int = 40, rk: int = 16,
            ncycle: int = 10, npow: int = 10, nals: int = 10, node_ncycle: int | None = None):
    """Solve H = sum_i (p_i^2 + q_i^2)/2 + lam sum_{i<D-1} (q_i^2 q_{i+1} - q_{i+1}^3/3)
    on the tree (0 1) (2 3) ... / top.  Returns (top eigenvalues, info)."""
    if D % 2:
        raise ValueError("the tree pairs the modes: D must be even")
    p2, q1, q2, q3 = H.ho_p2(n), H.ho_q_power(n, 1), H.ho_q_power(n, 2), H.ho_q_power(n, 3)
    # layer 1: one-mode operators and their eigenbases
    single, vecs, evals = [], [], []
    for i in range(D):
        h = 0.5 * p2 + 0.5 * q2 - ((lam / 3.0) * q3 if i >= 1 else 0.0)
        w, V = np.linalg.eigh(h)
        for j in range(n):
            if V[np.argmax(np.abs(V[:, j])), j] < 0:
                V[:, j] = -V[:, j]
        single.append(h)
        vecs.append(V)
        evals.append(w)
    tq1 = [V.T @ q1 @ V for V in vecs]
    tq2 = [V.T @ q2 @ V for V in vecs]
    # layer 2: the pair nodes (a two-mode vector of rank n already spans the
    # node, so the node rank is min(rk, n))
    npair = D // 2
    rk2 = min(rk, n)
    pairs = []
    for pi in range(npair):
        a, b = 2 * pi, 2 * pi + 1
        eig_ops = [np.diag(evals[a]), np.diag(evals[b])]
        terms = [(1.0, {0: eig_ops[0]}), (1.0, {1: eig_ops[1]}), (lam, {0: tq2[a], 1: tq1[b]})]
        hl = H.build_hoplist([n, n], terms, eig_ops)
        base, coef, eigv, hist = _node_states(hl, keep, rk2, node_ncycle or ncycle, npow, nals)
        pairs.append({"modes": (a, b), "base": base, "coef": coef, "eigv": eigv, "hist": hist})
    # layer 3: pair eigenvalues as eigen operators, couplings between pairs
    # carried into the pair bases (UpdateOperMat on the mode inside the pair)
    def carried(pi, mode_in_pair, X):
        pr = pairs[pi]
        packed = H.pack(X)
        out = IT.update_opermat(mode_in_pair + 1, pr["base"], pr["coef"], [n, n], rk2, keep, packed[None, :])
        return H.unpack(out[0], keep)

    eig_ops = [np.diag(pr["eigv"]) for pr in pairs]
    terms = [(1.0, {pi: eig_ops[pi]}) for pi in range(npair)]
    for i in range(D - 1):
        pa, pb = i // 2, (i + 1) // 2
        if pa == pb:
            continue  # inside a pair: already in the node Hamiltonian
        terms.append((lam, {pa: carried(pa, i % 2, tq2[i]), pb: carried(pb, (i + 1) % 2, tq1[i + 1])}))
    top = H.build_hoplist([keep] * npair, terms, eig_ops)
    _, _, eigv, _, hist = solver.solve(top, top_nev, rk, ncycle, npow, nals)
    return eigv, {"pairs": [{"eigv": p["eigv"], "last_rms": p["hist"][-1]} for p in pairs], "top_last_rms": hist[-1]}


def _modes(ops) -> frozenset:
    return frozenset(ops.keys())


def mode_tree(single, terms, layers, keep, rk: int, ncycle: int, npow: int, nals: int, log=None):
    """General multilayer walk (src/MLmain.f90:96-141) for a Hamiltonian given
    as primitive-basis terms [(coef, {mode: operator})].

    * Layer 1: each primitive mode's one-mode terms are diagonalised
      (HamilSetup); every multi-mode term's factor on the mode is carried into
      that eigenbasis.
    * Each later layer groups the previous layer's nodes (``layers``: one
      list of groups per layer, a group = child node indices; the last layer
      has one group, the top).  A node's Hamiltonian is its children's
      eigenvalues as diagonal operators plus every term whose modes lie in the
      node but in no single child, as the product of its children's carried
      factors.  The node is solved by the solver loop (spectral range, GPU
      power cycles) for ``keep[layer]`` states at rank min(rk, smallest child
      basis) when the node has two children (such a rank spans the node),
      else rk.
    * Terms reaching outside the node are carried into its basis: their
      factor on the node is <Q_j| prod over its children of the children's
      factors |Q_i> (UpdateH / UpdateOperMat, src/Updater.f90:53-151), one
      getqhqcpp_ call per distinct product.

    Returns (top eigenvalues, info)."""
    D = len(single)
    # layer 1
    nodes = []
    for m in range(D):
        h = sum(c * ops[m] for c, ops in terms if _modes(ops) == {m})
        w, V = np.linalg.eigh(h)
        for j in range(V.shape[1]):
            if V[np.argmax(np.abs(V[:, j])), j] < 0:
                V[:, j] = -V[:, j]
        fac = {t: V.T @ ops[m] @ V for t, (c, ops) in enumerate(terms) if m in ops and len(ops) > 1}
        nodes.append({"prims": frozenset([m]), "evals": w, "factors": fac})
    info = {"layers": []}
    for li, groups in enumerate(layers):
        nxt = []
        linfo = []
        for g in groups:
            ch = [nodes[c] for c in g]
            prims = frozenset().union(*[c["prims"] for c in ch])
            sizes = [c["evals"].size for c in ch]
            eig_ops = [np.diag(c["evals"]) for c in ch]
            node_terms = [(1.0, {i: eig_ops[i]}) for i in range(len(ch))]
            for t, (c, ops) in enumerate(terms):
                mt = _modes(ops)
                if not mt <= prims or any(mt <= cc["prims"] for cc in ch):
                    continue
                node_terms.append((c, {i: cc["factors"][t] for i, cc in enumerate(ch) if mt & cc["prims"]}))
            hl = H.build_hoplist(sizes, node_terms, eig_ops)
            nev = keep[li]
            rank = min(rk, min(sizes)) if len(ch) == 2 else rk
            base, coef, eigv, _, hist = solver.solve(hl, nev, rank, ncycle, npow, nals)
            node = {"prims": prims, "evals": eigv, "factors": {}}
            if li < len(layers) - 1:
                cache = {}
                for t, (c, ops) in enumerate(terms):
                    mt = _modes(ops)
                    if not (mt & prims) or mt <= prims:
                        continue
                    parts = {i: cc["factors"][t] for i, cc in enumerate(ch) if mt & cc["prims"]}
                    key = tuple((i, parts[i].tobytes()) for i in sorted(parts))
                    if key not in cache:
                        one = H.build_hoplist(sizes, [(1.0, parts)])
                        cache[key] = IT.qhq(base, coef, sizes, rank, nev, one)
                    node["factors"][t] = cache[key]
            nxt.append(node)
            linfo.append({"modes": sorted(prims), "terms": len(node_terms), "last_rms": hist[-1] if hist else None,
                          "carried": len(node["factors"]), "lowest": float(eigv[0])})
            if log:
                log(f"layer {li + 2} node {sorted(prims)}: {len(node_terms)} terms, E0 {eigv[0]:.6f}")
        nodes = nxt
        info["layers"].append(linfo)
    return nodes[0]["evals"], info


def qff_tree(D: int = 24, n: int = 8, seed: int = 3, keep_pair: int = 24, keep_group: int = 48, top_nev: int = 100,
             rk: int = 30, ncycle: int = 10, npow: int = 15, nals: int = 15, log=None):
    """The benchmark's three-layer tree for a synthetic quartic force field
    (hoplist.qff_terms): modes in pairs (0 1)(2 3)..., pairs of pairs, one top
    node over all groups of four."""
    if D % 4:
        raise ValueError("the three-layer tree groups modes in fours: D must be a multiple of 4")
    _, single, terms = H.qff_terms(D, n, seed)
    layers = [[[2 * i, 2 * i + 1] for i in range(D // 2)], [[2 * i, 2 * i + 1] for i in range(D // 4)],
              [list(range(D // 4))]]
    return mode_tree(single, terms, layers, [keep_pair, keep_group, top_nev], rk, ncycle, npow, nals, log=log)
