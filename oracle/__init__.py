"""CPU oracle for the single-phase finite-volume right-hand side.

TEST INFRASTRUCTURE ONLY.  Nothing in ``jaxfluids_gb300`` imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU baseline
leg of ``bench.py`` use it, and only to check or time against, never as
the thing measured or shipped.
"""
