"""CPU oracle for the xkep-cae assembly hot path.  TEST INFRASTRUCTURE ONLY.

This package restates, in vectorised NumPy, the reference algorithms that the
GPU kernels implement:

* ``oracle.beam``     - CR Timoshenko beam f_int / K_T
  (``xkep_cae/elements/_beam_cr.py``, ``xkep_cae/elements/_beam_assembly.py``)
* ``oracle.contact``  - AABB broadphase and candidate filters, segment-segment
  closest point, contact frame transport, active-set hysteresis, Huber normal
  force, Coulomb return mapping, and the contact / friction tangents
  (``xkep_cae/contact/...``)

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the parity reference or the timed CPU
baseline.  The product path (``xkgpu``) never imports it.

The oracle is pinned to the reference by golden vectors produced by running
the reference itself (``tests/golden/make_golden.py``), checked in
``tests/test_oracle_golden.py``.
"""
