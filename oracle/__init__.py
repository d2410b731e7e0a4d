"""CPU oracle for the VMC inner loop — TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy / torch-CPU FP64 code, the algorithm of
the reference's VMC hot path (sjdu10/vmc_torch): configuration encodings,
nearest-neighbour edges, the exchange-or-hop Metropolis proposal, Slater and
neural-backflow amplitudes, the spinful Fermi-Hubbard connected set with
symmray hop phases, local energies, log-derivatives, minSR and the
autocorrelation estimators.  Every function cites the reference file:line it
follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import this package, and only
as the checker or as the timed CPU baseline.  The product path
(``vmc_torch_gb300``) never imports it and has no CPU fallback.

Parity pins: the oracle is checked against golden vectors generated by the
reference's own code (``tests/golden/make_golden.py``, run in a container where
the reference sources are importable under import shims) and against the
reference's shipped example data (4x2 Hubbard checkpoints and energy history).
"""
