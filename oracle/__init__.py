"""CPU oracle: a float64 NumPy restatement of kUPS's particle-interaction path.

TEST INFRASTRUCTURE ONLY. Nothing in the ``kups_gb300`` package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use it, and there only as the checker (or as the timed CPU
baseline), never as the thing measured or shipped.

Parity is pinned against the reference's own known-answer tests
(``tests/test_oracle_golden.py``): the NaCl Madelung constant
(test/potential/test_ewald.py:53-56,272-335), the analytic Lennard-Jones pair
energies (test/potential/test_lennard_jones.py:172-289), the brute-force and
periodic-image neighbour-list cases (test/core/test_neighborlist.py:678-1221)
and the velocity-Verlet drift / reversibility bounds
(test/md/test_integrators.py:457-526).  The reference itself (JAX 0.10) cannot
be imported in this environment, so those tests' literal inputs and expected
values are the anchor.
"""
