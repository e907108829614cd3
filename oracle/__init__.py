"""
CPU oracle for the GFN1/GFN2-xTB single-point path.

TEST INFRASTRUCTURE ONLY. Nothing in the ``dxtb_gb300`` package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, and only as the checker or the timed CPU reference.

``xtb_oracle`` is a float64 restatement (PyTorch on the CPU, for autograd
forces) of the dxtb reference path; every function cites the reference file
and lines it follows. Its parity is pinned by the reference's own fixtures
(see ``tests/test_oracle_pins.py``).
"""
