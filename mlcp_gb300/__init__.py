"""GB300-native implementation of MLCP's GPU power-iteration hot path.

The compute path is the C-ABI library ``libmlcp_gb300.so`` (hand-written
CUDA for sm_103a, built in-tree by :mod:`mlcp_gb300.build`).  This package
mirrors the reference's operator interface on the host:

* :mod:`mlcp_gb300.als` — explicit-target ALS rank reduction (alscpp_);
* :mod:`mlcp_gb300.intertwine` — one intertwined power cycle (intertwinecpp_);
* :mod:`mlcp_gb300.hoplist` — Hamiltonian operator lists (HopList);
* :mod:`mlcp_gb300.workloads` — seeded synthetic benchmark inputs.

Importing the package does not load the library; the first compute call
builds (if needed) and loads it, and raises if that is impossible.
"""

__all__ = ["als", "hoplist", "workloads", "build"]
