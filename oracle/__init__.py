"""CPU oracle for the SG-MCMC hot path -- TEST INFRASTRUCTURE ONLY.

This package restates the reference (jax_sgmc 0.1.5) arithmetic on the CPU
with numpy, function by function, each citing the reference file:line it
follows.  The CUDA path is checked against it: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and
``--impl reference`` arm) may import it.  The product (the ``gbsgmc``
package and ``libgbsgmc.so``) never calls it.

Pinning: the index stream is checked against numpy's own
``Generator.choice`` (the reference's call, numpy_loader.py:382-389); the
Philox4x32-10 restatement against the Random123 known-answer vectors; the
potential against the reference's known-answer tests (tests/test_potential.py)
restated in ``tests/test_oracle.py``; the scheduler against
tests/test_scheduler.py.  Trajectory-level arithmetic (integrator steps,
RMSprop values, swap) is pinned by no reference test and is checked by
construction against the reference source, with fixtures in tests/golden/.
"""
