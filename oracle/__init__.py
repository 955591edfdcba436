"""CPU oracle for the multislice ptychography hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain NumPy/SciPy, the reference algorithm of pypty's
``multislice_core`` / ``objective.loss_and_direction`` / ``fft`` path for the flag set the
GPU path supports. It is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it. The GPU product path never imports or
calls anything here.

Parity pin: ``tests/test_oracle_golden.py`` checks this restatement against golden vectors
produced by running the reference's own NumPy path (``tests/golden/make_golden.py``).
"""
