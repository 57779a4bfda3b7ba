"""Minimal stand-in for the one Cirq symbol mpsim/core_test.py imports.

Test infrastructure only (Cirq is not installed).  core_test.py:22 imports
``cirq.qis.density_matrix_from_state_vector``; ``qis`` restates it.
"""
from . import qis  # noqa: F401
