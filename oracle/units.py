"""Unit system of the reference (ASE-consistent: Angstrom, eV, amu).

The constant table (src/kups/core/constants.py:26-76, CODATA 2014 values as used by ASE) is
data shared by the library and the oracle; it is kept once, in kups_gb300/units.py, and the
oracle reads it from there.  Test infrastructure: imported by tests, smoke() and bench.py's
CPU legs only.
"""

from kups_gb300.units import (  # noqa: F401
    BAR,
    BOHR,
    BOLTZMANN_CONSTANT,
    EPSILON_0,
    FEMTO_SECOND,
    HARTREE,
    HBAR,
    KILO_CALORIE,
    KILO_JOULE,
    METER,
    MOL,
    PASCAL,
    SECOND,
    TO_STANDARD_UNITS,
)
