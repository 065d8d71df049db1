"""CPU oracle for the structured-grid stencil path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import anything from here, and
only as the checker or the timed CPU baseline.  The product path
(``npbench_gb300``) never imports this package: it runs the CUDA kernels of
``libnpbgb.so`` and raises when that library is missing.

Two restatements of NPBench's NumPy kernels live here:

* ``stencils_np``  -- NumPy, one ufunc per reference operator, same evaluation
  order; bit-identical to the reference by construction.
* ``stencils.c``   -- plain C (``-ffp-contract=off``), optionally OpenMP; the
  same per-point operation order, so it is bit-identical too.  Loaded through
  ``oracle.cref``.

Both are pinned against golden vectors produced by importing the reference's
own NumPy modules (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.
"""
