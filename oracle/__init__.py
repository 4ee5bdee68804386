"""Oracle for torchfsm's Fourier-spectral ETD time-stepping path.

TEST INFRASTRUCTURE ONLY. Nothing in the product imports this package: only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline``
leg and its ``--impl reference`` arm) may import it, and only to compare
results against it or as the timed CPU restatement of the reference.

``oracle.spectral`` restates, in numpy FP64 (complex128, full C2C spectra),
the reference's mesh symbols, nonlinear cores, exponential-integrator
coefficients and the ``integrate`` loop. Each function cites the reference
file:line it follows (paths relative to the torchfsm project root).

Parity pin: the restatement is checked against golden vectors produced by the
reference itself (``tests/golden/make_golden.py`` imports torchfsm 0.0.4 and
runs it in float64); ``tests/test_oracle_golden.py`` asserts agreement to
~1e-10 relative.
"""
