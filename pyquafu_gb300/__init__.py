"""pyquafu_gb300: GB300 (sm_103a) statevector engine for pyquafu.

Drop-in for the gate-application hot path behind ``quafu.simulators`` and the
``qfvm`` pybind module (see ``pyquafu_gb300.qfvm``), plus device-resident
states, compiled plans, Pauli expectations, seeded sampling and adjoint
gradients.
"""

from ._native import QfvmError, launch_count  # noqa: F401
from .builder import build  # noqa: F401

__version__ = "0.1.0"
