"""CPU oracle for the lime open-system propagator (TEST INFRASTRUCTURE ONLY).

This package restates, in NumPy, the algorithm of the reference solvers in
``lime/oqs.py``, ``lime/phys.py`` and ``lime/superoperator.py`` of
binggu56/lime.  It is the checker for the CUDA path and the timed CPU
baseline; nothing in ``lime_gb300`` imports it.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may use it.

Parity of this restatement is pinned against golden vectors produced by
running the reference itself (``tests/golden/make_golden.py``); the check
lives in ``tests/test_oracle_golden.py``.

Modules
-------
lindblad   RK4 Lindblad propagation and quantum-regression correlations
           (``lime/oqs.py:706-800, 1117-1331, 1590-1800``; ``lime/phys.py:636-649``).
superop    Liouville-space (row-major vec) superoperators and the eigen-series
           solver (``lime/superoperator.py:30-271, 456-773``).
redfield   Bloch-Redfield tensor and RK4 on vec(rho)
           (``lime/oqs.py:40-371, 373-472, 528-579``).
spectra    FFT with the reference sign convention (``lime/fft.py:9-56``).
pool       Multi-process timing harness for the CPU baseline.
"""
