"""CPU oracle for the matrix-product hot path (test infrastructure only).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and its
``--impl reference`` arm) may import it.  The shipped path lives in
``syngular_gb300`` and runs on the GPU through the C-ABI library.

* ``tt_fp64``  -- numpy FP64 restatement of Syngular's MPS/MPO algorithms
  (each function cites the reference ``file:line`` it follows) plus the
  TT-SVD rounding the GPU path adds, with seeded workload generators.
* ``ref_shim`` -- imports the unmodified Python reference as ``syngular`` in a
  development container (stubs for its unused imports, numpy-2 shims); used
  only by ``tests/golden/make_golden.py`` to pin this oracle with fixtures.

Parity status: QR-truncation ``>>``, ``@``, ``+``, ``|``, ``decompose`` and
orthonormalisation are pinned by fixtures generated from the reference.  The
TT-SVD rounding has no reference counterpart ("parity unpinned" for that
function only); it is checked against dense SVD truncation identities.
"""
