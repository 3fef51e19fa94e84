"""GB300-native discrete adjoint of controlled explicit Runge-Kutta integration.

The compute path is libva_gb300.so (hand-written CUDA for sm_103a behind the C
ABI of include/va.h).  This package is the Python host layer over that ABI:
`Solver` for batches and the reference-style single-instance facade in
`driver` (Driver, runge_kutta, setCostGradients, adjointSolve, ...).
"""
from ._lib import LIB_PATH, STATUS_NAMES, VaError, load  # noqa: F401
from .autograd import odeint_adjoint  # noqa: F401
from .solver import Solver  # noqa: F401
